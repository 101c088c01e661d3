// krylov.cu -- see krylov.cuh.
#include <stdint.h>

#include "krylov.cuh"

namespace icep {

namespace {

constexpr int TPB = 256;

__device__ __forceinline__ long real_index(const Grid &g, unsigned t) {
  int i, j, k;
  real_ijk(g, t, i, j, k);
  return gidx(g, i, j, k);
}

// Grid-stride partial dots; fixed grid size and fixed reduction order make the
// result independent of timing (deterministic).
template <typename R>
__global__ void k_dots(Grid g, const R *a0, const R *b0, const R *a1, const R *b1, int n, double *partials) {
  double s0 = 0.0, s1 = 0.0;
  const unsigned N = (unsigned)g.nreal();
  for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < N; t += gridDim.x * blockDim.x) {
    const long im = real_index(g, t);
    s0 += (double)a0[im] * (double)b0[im];
    if (n > 1) s1 += (double)a1[im] * (double)b1[im];
  }
  __shared__ double red[2][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
  }
  if (lane == 0) {
    red[0][wid] = s0;
    red[1][wid] = s1;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += red[threadIdx.x][w];
    partials[blockIdx.x * 2 + threadIdx.x] = v;
  }
}

__global__ void k_dots_final(const double *partials, int nblocks, int n, double *scal, int slot) {
  __shared__ double red[2][32];
  double s0 = 0.0, s1 = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    s0 += partials[2 * b];
    s1 += partials[2 * b + 1];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
  }
  if (lane == 0) {
    red[0][wid] = s0;
    red[1][wid] = s1;
  }
  __syncthreads();
  if (threadIdx.x < n) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += red[threadIdx.x][w];
    scal[slot + threadIdx.x] = v;
  }
}

template <typename R>
__global__ void k_sum(Grid g, const R *a, double *partials, int absval) {
  // the thread's terms in the field type, the block and grid sums in FP64
  R t0 = R(0);
  const unsigned N = (unsigned)g.nreal();
  for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < N; t += gridDim.x * blockDim.x) {
    const R v = a[real_index(g, t)];
    t0 += absval ? fabs(v) : v;
  }
  __shared__ double red[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) t0 += __shfl_down_sync(0xffffffffu, t0, o);
  if (lane == 0) red[wid] = (double)t0;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += red[w];
    partials[blockIdx.x * 2] = v;
    partials[blockIdx.x * 2 + 1] = 0.0;
  }
}

#define RTID ((unsigned)(blockIdx.x * blockDim.x + threadIdx.x))

template <typename R>
__global__ void k_bicg_p(Grid g, R *p, const R *r, const R *v, R beta, R w) {
  const unsigned t = RTID;
  if (t >= (unsigned)g.nreal()) return;
  const long im = real_index(g, t);
  p[im] = r[im] + beta * (p[im] - w * v[im]);
}

template <typename R>
__global__ void k_bicg_s(Grid g, R *sv, const R *r, const R *v, double rho, const double *scal) {
  const unsigned t = RTID;
  if (t >= (unsigned)g.nreal()) return;
  const R alpha = (R)(rho / scal[S_R0V]);
  const long im = real_index(g, t);
  sv[im] = r[im] - alpha * v[im];
}

template <typename R>
__global__ void k_bicg_xr(Grid g, R *x, R *r, const R *y, const R *z, const R *sv, const R *tv, double rho,
                          const double *scal) {
  const unsigned t = RTID;
  if (t >= (unsigned)g.nreal()) return;
  const R alpha = (R)(rho / scal[S_R0V]);
  const double tt = scal[S_TT];
  const R w = (R)((tt > 0.0) ? scal[S_TS] / tt : 0.0);
  const long im = real_index(g, t);
  x[im] += alpha * y[im] + w * z[im];
  r[im] = sv[im] - w * tv[im];
}

template <typename R>
__global__ void k_copy_real(Grid g, const R *x, R *y) {
  const unsigned t = RTID;
  if (t >= (unsigned)g.nf()) return;
  const unsigned k = t % (unsigned)g.nzp;
  y[t] = (k < (unsigned)g.nz) ? x[t] : R(0);
}

template <typename R>
__global__ void k_sub_real(Grid g, const R *b, const R *tv, R *r) {
  const unsigned t = RTID;
  if (t >= (unsigned)g.nreal()) return;
  const long im = real_index(g, t);
  r[im] = b[im] - tv[im];
}

template <typename R>
__global__ void k_sub_mean(Grid g, R *a, const double *scal, int slot) {
  const unsigned t = RTID;
  if (t >= (unsigned)g.nreal()) return;
  const R m = (R)(scal[slot] / (double)g.nreal());
  const long im = real_index(g, t);
  a[im] -= m;
}

__global__ void k_f2d(long n, const float *x, double *y) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) y[t] = (double)x[t];
}
__global__ void k_d2f(long n, const double *x, float *y) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) y[t] = (float)x[t];
}
// Conversions that read or write host memory mapped into the device's
// address space: 16-byte accesses (two values per thread and iteration) and
// a grid of a few blocks per SM striding over the array, so that many
// requests cross the CPU-GPU link at once.
__global__ void k_d2f_link(long n2, const double2 *__restrict__ x, float2 *__restrict__ y) {
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n2; t += (long)gridDim.x * blockDim.x) {
    const double2 v = x[t];
    y[t] = make_float2((float)v.x, (float)v.y);
  }
}
__global__ void k_f2d_link(long n2, const float2 *__restrict__ x, double2 *__restrict__ y) {
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n2; t += (long)gridDim.x * blockDim.x) {
    const float2 v = x[t];
    y[t] = make_double2((double)v.x, (double)v.y);
  }
}
__global__ void k_copy_link(long n2, const double2 *__restrict__ x, double2 *__restrict__ y) {
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n2; t += (long)gridDim.x * blockDim.x) y[t] = x[t];
}
// element-wise over all n values (k-space arrays included)
__global__ void k_scale_d2f_all(long n, const double *x, float *y, double a) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) y[t] = (float)(a * x[t]);
}
__global__ void k_add_f2d_all(long n, const float *x, double *y, double a) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) y[t] += a * (double)x[t];
}
__global__ void k_axpby_all(long n, const double *x, double *y, double a, double b) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) y[t] = a * x[t] + b * y[t];
}

__global__ void k_add_f2d(Grid g, const float *x, double *y, double a) {
  const unsigned t = RTID;
  if (t >= (unsigned)g.nreal()) return;
  const long im = real_index(g, t);
  y[im] += a * (double)x[im];
}
__global__ void k_scale_d2f(Grid g, const double *x, float *y, double a) {
  const unsigned t = RTID;
  if (t >= (unsigned)g.nf()) return;
  const unsigned k = t % (unsigned)g.nzp;
  y[t] = (k < (unsigned)g.nz) ? (float)(a * x[t]) : 0.0f;
}

}  // namespace

template <typename R>
void dots(const Grid &g, const R *a0, const R *b0, const R *a1, const R *b1, int n, double *partials, double *scal,
          int slot, cudaStream_t s) {
  count_launch(fld<R>(g, ndistinct(a0, b0, n > 1 ? a1 : nullptr, n > 1 ? b1 : nullptr)));
  k_dots<R><<<DOT_BLOCKS, DOT_TPB, 0, s>>>(g, a0, b0, a1, b1, n, partials);
  count_launch();
  k_dots_final<<<1, 256, 0, s>>>(partials, DOT_BLOCKS, n, scal, slot);
}
template <typename R>
void sum_real(const Grid &g, const R *a, double *partials, double *scal, int slot, cudaStream_t s) {
  count_launch(fld<R>(g, 1));
  k_sum<R><<<DOT_BLOCKS, DOT_TPB, 0, s>>>(g, a, partials, 0);
  count_launch();
  k_dots_final<<<1, 256, 0, s>>>(partials, DOT_BLOCKS, 1, scal, slot);
}
template <typename R>
void sum_abs_real(const Grid &g, const R *a, double *partials, double *scal, int slot, cudaStream_t s) {
  count_launch(fld<R>(g, 1));
  k_sum<R><<<DOT_BLOCKS, DOT_TPB, 0, s>>>(g, a, partials, 1);
  count_launch();
  k_dots_final<<<1, 256, 0, s>>>(partials, DOT_BLOCKS, 1, scal, slot);
}
template <typename R>
void bicg_p(const Grid &g, R *p, const R *r, const R *v, double beta, double w, cudaStream_t s) {
  count_launch(fld<R>(g, 4));
  k_bicg_p<R><<<div_up(g.nreal(), TPB), TPB, 0, s>>>(g, p, r, v, (R)beta, (R)w);
}
template <typename R>
void bicg_s(const Grid &g, R *sv, const R *r, const R *v, double rho, const double *scal, cudaStream_t s) {
  count_launch(fld<R>(g, 3));
  k_bicg_s<R><<<div_up(g.nreal(), TPB), TPB, 0, s>>>(g, sv, r, v, rho, scal);
}
template <typename R>
void bicg_xr(const Grid &g, R *x, R *r, const R *y, const R *z, const R *sv, const R *t, double rho,
             const double *scal, cudaStream_t s) {
  count_launch(fld<R>(g, 7));
  k_bicg_xr<R><<<div_up(g.nreal(), TPB), TPB, 0, s>>>(g, x, r, y, z, sv, t, rho, scal);
}
template <typename R>
void copy_real(const Grid &g, const R *x, R *y, cudaStream_t s) {
  count_launch(fld<R>(g, 2));
  k_copy_real<R><<<div_up(g.nf(), TPB), TPB, 0, s>>>(g, x, y);
}
template <typename R>
void sub_real(const Grid &g, const R *b, const R *t, R *r, cudaStream_t s) {
  count_launch(fld<R>(g, 3));
  k_sub_real<R><<<div_up(g.nreal(), TPB), TPB, 0, s>>>(g, b, t, r);
}
template <typename R>
void sub_mean(const Grid &g, R *a, const double *scal, int slot, cudaStream_t s) {
  count_launch(fld<R>(g, 2));
  k_sub_mean<R><<<div_up(g.nreal(), TPB), TPB, 0, s>>>(g, a, scal, slot);
}
void convert_f2d(long n, const float *x, double *y, cudaStream_t s) {
  count_launch(12.0 * n);
  k_f2d<<<div_up(n, TPB), TPB, 0, s>>>(n, x, y);
}
void convert_d2f(long n, const double *x, float *y, cudaStream_t s) {
  count_launch(12.0 * n);
  k_d2f<<<div_up(n, TPB), TPB, 0, s>>>(n, x, y);
}
namespace {
bool link_ok(long n, const void *a, const void *b) {
  return (n % 2) == 0 && ((uintptr_t)a % 16) == 0 && ((uintptr_t)b % 16) == 0;
}
unsigned link_blocks(long n2) {
  const long want = (n2 + TPB - 1) / TPB, cap = 152L * 8;
  return (unsigned)(want < cap ? want : cap);
}
}  // namespace
void link_d2f(long n, const double *x, float *y, cudaStream_t s) {
  if (!link_ok(n, x, y)) return convert_d2f(n, x, y, s);
  count_launch(12.0 * n);
  k_d2f_link<<<link_blocks(n / 2), TPB, 0, s>>>(n / 2, reinterpret_cast<const double2 *>(x),
                                                 reinterpret_cast<float2 *>(y));
}
void link_f2d(long n, const float *x, double *y, cudaStream_t s) {
  if (!link_ok(n, x, y)) return convert_f2d(n, x, y, s);
  count_launch(12.0 * n);
  k_f2d_link<<<link_blocks(n / 2), TPB, 0, s>>>(n / 2, reinterpret_cast<const float2 *>(x),
                                                 reinterpret_cast<double2 *>(y));
}
void link_copy(long n, const double *x, double *y, cudaStream_t s) {
  if (!link_ok(n, x, y)) {
    cudaMemcpyAsync(y, x, sizeof(double) * n, cudaMemcpyDefault, s);
    return;
  }
  count_launch(16.0 * n);
  k_copy_link<<<link_blocks(n / 2), TPB, 0, s>>>(n / 2, reinterpret_cast<const double2 *>(x),
                                                  reinterpret_cast<double2 *>(y));
}
void scale_d2f_all(long n, const double *x, float *y, double a, cudaStream_t s) {
  count_launch(12.0 * n);
  k_scale_d2f_all<<<div_up(n, TPB), TPB, 0, s>>>(n, x, y, a);
}
void add_f2d_all(long n, const float *x, double *y, double a, cudaStream_t s) {
  count_launch(20.0 * n);
  k_add_f2d_all<<<div_up(n, TPB), TPB, 0, s>>>(n, x, y, a);
}
void axpby_all(long n, const double *x, double *y, double a, double b, cudaStream_t s) {
  count_launch(24.0 * n);
  k_axpby_all<<<div_up(n, TPB), TPB, 0, s>>>(n, x, y, a, b);
}
void add_f2d(const Grid &g, const float *x, double *y, double a, cudaStream_t s) {
  count_launch(fld<float>(g, 1) + fld<double>(g, 2));
  k_add_f2d<<<div_up(g.nreal(), TPB), TPB, 0, s>>>(g, x, y, a);
}
void scale_d2f(const Grid &g, const double *x, float *y, double a, cudaStream_t s) {
  count_launch(fld<double>(g, 1) + fld<float>(g, 1));
  k_scale_d2f<<<div_up(g.nf(), TPB), TPB, 0, s>>>(g, x, y, a);
}

#define KRY_INST(R)                                                                                              \
  template void dots<R>(const Grid &, const R *, const R *, const R *, const R *, int, double *, double *, int, \
                        cudaStream_t);                                                                           \
  template void sum_real<R>(const Grid &, const R *, double *, double *, int, cudaStream_t);                     \
  template void sum_abs_real<R>(const Grid &, const R *, double *, double *, int, cudaStream_t);                 \
  template void bicg_p<R>(const Grid &, R *, const R *, const R *, double, double, cudaStream_t);                \
  template void bicg_s<R>(const Grid &, R *, const R *, const R *, double, const double *, cudaStream_t);        \
  template void bicg_xr<R>(const Grid &, R *, R *, const R *, const R *, const R *, const R *, double,           \
                           const double *, cudaStream_t);                                                        \
  template void copy_real<R>(const Grid &, const R *, R *, cudaStream_t);                                        \
  template void sub_real<R>(const Grid &, const R *, const R *, R *, cudaStream_t);                              \
  template void sub_mean<R>(const Grid &, R *, const double *, int, cudaStream_t);

KRY_INST(double)
KRY_INST(float)

}  // namespace icep
