// refine.cu -- float-float kernels of the MIXED Poisson refinement (see
// refine.cuh). Every kernel is one pass over its vectors with 16-byte
// (complex float-float) or 8-byte (real float-float) accesses; none executes
// FP64 arithmetic per element except rf_to_f64 (field read-back only).
#include <math.h>

#include <vector>

#include "krylov.cuh"
#include "kspace.cuh"
#include "refine.cuh"

namespace icep {

namespace {

constexpr int TPB = 256;

// a complex float-float number as float4 (re.hi, re.lo, im.hi, im.lo)
__device__ __forceinline__ dfl re_of(float4 v) { return dfl(v.x, v.y); }
__device__ __forceinline__ dfl im_of(float4 v) { return dfl(v.z, v.w); }
__device__ __forceinline__ float4 pack(dfl re, dfl im) { return make_float4(re.hi, re.lo, im.hi, im.lo); }

// (ar + i ai)(br + i bi) in float-float
__device__ __forceinline__ void cmul_df(dfl ar, dfl ai, dfl br, dfl bi, dfl &cr, dfl &ci) {
  cr = ar * br - ai * bi;
  ci = ar * bi + ai * br;
}

__global__ void k_rf_from_f32(long n, const float *__restrict__ a, float2 *__restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) out[t] = make_float2(a[t], 0.f);
}

// scale_dev (if given) replaces scale: a factor formed on the device
__global__ void k_rf_to_f32(long n, const float2 *__restrict__ a, float *__restrict__ out, float scale,
                            const float *scale_dev) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) {
    const float sc = scale_dev ? *scale_dev : scale;
    const float2 v = a[t];
    out[t] = __fadd_rn(v.x, v.y) * sc;
  }
}

__global__ void k_rf_to_f64(long n, const float2 *__restrict__ a, double *__restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) {
    const float2 v = a[t];
    out[t] = (double)v.x + (double)v.y;
  }
}

// a_dev (if given: hi, lo) replaces a
__global__ void k_rf_add_f32(long n, const float *__restrict__ d, float2 *__restrict__ x, dfl a,
                             const float2 *a_dev) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) {
    if (a_dev) a = dfl(a_dev->x, a_dev->y);
    const float2 v = x[t];
    const dfl r = dfl(v.x, v.y) + a * d[t];
    x[t] = make_float2(r.hi, r.lo);
  }
}

// x <- 2 x - xp (the linear extrapolation in time) and xp <- x, in place
__global__ void k_rf_extrapolate_shift(long n, float2 *__restrict__ x, float2 *__restrict__ xp) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) {
    const float2 a = x[t], b = xp[t];
    const dfl r = dfl(2.f * a.x, 2.f * a.y) - dfl(b.x, b.y);
    x[t] = make_float2(r.hi, r.lo);
    xp[t] = a;
  }
}

__global__ void k_rf_zero_if(long n, float2 *__restrict__ x, const double *flag) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n && *flag != 0.0) x[t] = make_float2(0.f, 0.f);
}

struct RfTab {
  const float4 *gd[3];
};

// mode t (complex index) -> (i, j, kz); grids hold at most 2^24 points
__device__ __forceinline__ void mode_ijk(const Grid &g, unsigned t, int &i, int &j, int &kz) {
  mode_ijk3(g, t, i, j, kz);
}

__global__ void k_rf_grad(Grid g, RfTab tab, const float4 *__restrict__ x, float4 *__restrict__ w0,
                          float4 *__restrict__ w1, float4 *__restrict__ w2) {
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (unsigned)g.nmodes()) return;
  int i, j, kz;
  mode_ijk(g, t, i, j, kz);
  const float4 a = x[t];
  const dfl ar = re_of(a), ai = im_of(a);
  const float4 m0 = tab.gd[0][i], m1 = tab.gd[1][j], m2 = tab.gd[2][kz];
  dfl cr, ci;
  cmul_df(re_of(m0), im_of(m0), ar, ai, cr, ci);
  w0[t] = pack(cr, ci);
  cmul_df(re_of(m1), im_of(m1), ar, ai, cr, ci);
  w1[t] = pack(cr, ci);
  cmul_df(re_of(m2), im_of(m2), ar, ai, cr, ci);
  w2[t] = pack(cr, ci);
}

// real point t -> padded index and the padded indices of its +x, +y, +z
// neighbours (periodic; sizes are powers of two)
__device__ __forceinline__ bool point_nbrs(const Grid &g, long tl, long &im, long &n0, long &n1, long &n2) {
  if (tl >= g.nreal()) return false;
  int i, j, k;
  real_ijk(g, (unsigned)tl, i, j, k);
  im = gidx(g, i, j, k);
  n0 = gidx(g, (i + 1) & (g.nx - 1), j, k);
  n1 = gidx(g, i, (j + 1) & (g.ny - 1), k);
  n2 = gidx(g, i, j, (k + 1) & (g.nz - 1));
  return true;
}

__device__ __forceinline__ dfl face(float a, float b) { return half_of(two_sum(a, b)); }

__global__ void k_rf_eps_face_mul(Grid g, float2 *__restrict__ w0, float2 *__restrict__ w1, float2 *__restrict__ w2,
                                  const float *__restrict__ eps) {
  long im, n0, n1, n2;
  if (!point_nbrs(g, (long)blockIdx.x * blockDim.x + threadIdx.x, im, n0, n1, n2)) return;
  const float e = eps[im];
  float2 *w[3] = {w0, w1, w2};
  const long nb[3] = {n0, n1, n2};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const float2 v = w[d][im];
    const dfl r = dfl(v.x, v.y) * face(e, eps[nb[d]]);
    w[d][im] = make_float2(r.hi, r.lo);
  }
}

__global__ void k_rf_eps_face_e(Grid g, float2 *__restrict__ w0, float2 *__restrict__ w1, float2 *__restrict__ w2,
                                const float *__restrict__ eps, dfl e0, dfl e1, dfl e2, int use) {
  long im, n0, n1, n2;
  if (!point_nbrs(g, (long)blockIdx.x * blockDim.x + threadIdx.x, im, n0, n1, n2)) return;
  const float e = eps[im];
  float2 *w[3] = {w0, w1, w2};
  const long nb[3] = {n0, n1, n2};
  const dfl ed[3] = {e0, e1, e2};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (!(use & (1 << d))) continue;
    const dfl r = face(e, eps[nb[d]]) * ed[d];
    w[d][im] = make_float2(r.hi, r.lo);
  }
}

template <bool ACC64>
__global__ void __launch_bounds__(DOT_TPB) k_rf_div_combine(Grid g, RfTab tab, const float4 *__restrict__ w0,
                                                             const float4 *__restrict__ w1, const float4 *__restrict__ w2,
                                                             int use, const float4 *__restrict__ base,
                                                             float4 *__restrict__ out, int mode, float prescale,
                                                             double post, double *__restrict__ partials,
                                                             const float *prescale_dev) {
  if (!ACC64 && prescale_dev) {  // the prescale formed on the device, post as the host forms it
    prescale = *prescale_dev;
    post = (1.0 / ((double)prescale * (double)prescale)) / (double)g.nreal();
  }
  const unsigned N = (unsigned)g.nmodes();
  const float4 *w[3] = {w0, w1, w2};
  float acc = 0.f;
  double acc64 = 0.0;
  for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < N; t += gridDim.x * blockDim.x) {
    int i, j, kz;
    mode_ijk(g, t, i, j, kz);
    const int idx[3] = {i, j, kz};
    dfl sr(0), si(0);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      if (!(use & (1 << d))) continue;
      const float4 m = tab.gd[d][idx[d]];
      const float4 v = w[d][t];
      // D^-_d = -conj(D^+_d) = (-re, im)
      dfl cr, ci;
      cmul_df(-re_of(m), im_of(m), re_of(v), im_of(v), cr, ci);
      sr += cr;
      si += ci;
    }
    const float4 b = base[t];
    dfl orr, oi;
    if (mode == RF_RESIDUAL) {
      orr = re_of(b) - sr;
      oi = im_of(b) - si;
    } else {
      orr = sr - re_of(b);
      oi = si - im_of(b);
      if (t == 0) orr = oi = dfl(0);
    }
    out[t] = pack(orr, oi);
    const int wt = read_weight(g, i, j, kz);
    if (wt == 0) continue;
    const float im = (wt == 1) ? 0.f : oi.hi;  // self-conjugate modes: real part only
    if (ACC64) {
      acc64 += (double)wt * ((double)orr.hi * (double)orr.hi + (double)im * (double)im);
    } else {
      const float xr = orr.hi * prescale, xi = im * prescale;
      acc = fmaf((float)wt, fmaf(xr, xr, xi * xi), acc);
    }
  }
  __shared__ double red[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (ACC64) {
    for (int o = 16; o > 0; o >>= 1) acc64 += __shfl_down_sync(0xffffffffu, acc64, o);
  } else {  // warp sums in FP32, one FP64 value per warp
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  }
  if (lane == 0) red[wid] = ACC64 ? acc64 : (double)acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) sum += red[q];
    partials[2 * blockIdx.x] = sum * post;
    partials[2 * blockIdx.x + 1] = 0.0;
  }
}

__global__ void k_rf_differs(long n, const unsigned long long *__restrict__ a,
                             const unsigned long long *__restrict__ b, int *flag) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n && a[t] != b[t]) *flag = 1;
}

inline unsigned nblk(long n) { return div_up(n, TPB); }

}  // namespace

int RefineTables::init(const Grid &g, cudaStream_t s) {
  const int n[3] = {g.nx, g.ny, g.hnz};
  std::vector<float4> h((size_t)(n[0] + n[1] + n[2]));
  size_t off = 0;
  for (int d = 0; d < 3; d++)
    for (int q = 0; q < n[d]; q++, off++) {
      const int kint = (d == 0) ? kx_of(g, q) : (d == 1) ? ky_of(g, q) : q;
      const long double k = (long double)g.wave[d] * kint;
      const long double a = 0.5L * (long double)g.dx * k;
      // D^+ = i k exp(i a) = (-k sin a, k cos a)
      const long double re = -k * sinl(a), im = k * cosl(a);
      const float rh = (float)re, ih = (float)im;
      h[off] = make_float4(rh, (float)(re - (long double)rh), ih, (float)(im - (long double)ih));
    }
  if (cudaMalloc(&mem, sizeof(float4) * h.size()) != cudaSuccess) return ICEP_ERR_CUDA;
  cudaMemcpyAsync(mem, h.data(), sizeof(float4) * h.size(), cudaMemcpyHostToDevice, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return ICEP_ERR_CUDA;
  float4 *b = static_cast<float4 *>(mem);
  gd[0] = b;
  gd[1] = b + n[0];
  gd[2] = b + n[0] + n[1];
  return ICEP_OK;
}

void RefineTables::free_all() {
  cudaFree(mem);
  mem = nullptr;
  gd[0] = gd[1] = gd[2] = nullptr;
}

static RfTab tab_of(const RefineTables &t) { return RfTab{{t.gd[0], t.gd[1], t.gd[2]}}; }

void rf_from_f32(long n, const float *a, dfl *out, cudaStream_t s) {
  count_launch(12.0 * n);
  k_rf_from_f32<<<nblk(n), TPB, 0, s>>>(n, a, reinterpret_cast<float2 *>(out));
}
void rf_to_f32(long n, const dfl *a, float *out, double scale, cudaStream_t s) {
  count_launch(12.0 * n);
  k_rf_to_f32<<<nblk(n), TPB, 0, s>>>(n, reinterpret_cast<const float2 *>(a), out, (float)scale, nullptr);
}
void rf_to_f32(long n, const dfl *a, float *out, const float *scale_dev, cudaStream_t s) {
  count_launch(12.0 * n);
  k_rf_to_f32<<<nblk(n), TPB, 0, s>>>(n, reinterpret_cast<const float2 *>(a), out, 1.f, scale_dev);
}
void rf_differs(long n, const double *a, const double *b, int *flag, cudaStream_t s) {
  cudaMemsetAsync(flag, 0, sizeof(int), s);
  count_launch(16.0 * n);
  k_rf_differs<<<nblk(n), TPB, 0, s>>>(n, reinterpret_cast<const unsigned long long *>(a),
                                       reinterpret_cast<const unsigned long long *>(b), flag);
}
void rf_to_f64(long n, const dfl *a, double *out, cudaStream_t s) {
  count_launch(16.0 * n);
  k_rf_to_f64<<<nblk(n), TPB, 0, s>>>(n, reinterpret_cast<const float2 *>(a), out);
}
void rf_add_f32(long n, const float *d, dfl *x, double a, cudaStream_t s) {
  count_launch(20.0 * n);
  k_rf_add_f32<<<nblk(n), TPB, 0, s>>>(n, d, reinterpret_cast<float2 *>(x), dfl::from_double(a), nullptr);
}
void rf_add_f32(long n, const float *d, dfl *x, const float2 *a_dev, cudaStream_t s) {
  count_launch(20.0 * n);
  k_rf_add_f32<<<nblk(n), TPB, 0, s>>>(n, d, reinterpret_cast<float2 *>(x), dfl(0), a_dev);
}
void rf_extrapolate_shift(long n, dfl *x, dfl *xp, cudaStream_t s) {
  count_launch(32.0 * n);
  k_rf_extrapolate_shift<<<nblk(n), TPB, 0, s>>>(n, reinterpret_cast<float2 *>(x), reinterpret_cast<float2 *>(xp));
}
void rf_zero_if(long n, dfl *x, const double *flag, cudaStream_t s) {
  count_launch();
  k_rf_zero_if<<<nblk(n), TPB, 0, s>>>(n, reinterpret_cast<float2 *>(x), flag);
}
void rf_grad(const Grid &g, const RefineTables &t, const dfl *x, dfl *w0, dfl *w1, dfl *w2, cudaStream_t s) {
  count_launch(fld<double>(g, 4));
  k_rf_grad<<<nblk(g.nmodes()), TPB, 0, s>>>(g, tab_of(t), reinterpret_cast<const float4 *>(x),
                                             reinterpret_cast<float4 *>(w0), reinterpret_cast<float4 *>(w1),
                                             reinterpret_cast<float4 *>(w2));
}
void rf_eps_face_mul(const Grid &g, dfl *w0, dfl *w1, dfl *w2, const float *eps, cudaStream_t s) {
  count_launch(fld<double>(g, 6) + fld<float>(g, 1));
  k_rf_eps_face_mul<<<nblk(g.nreal()), TPB, 0, s>>>(g, reinterpret_cast<float2 *>(w0), reinterpret_cast<float2 *>(w1),
                                                    reinterpret_cast<float2 *>(w2), eps);
}
void rf_eps_face_e(const Grid &g, dfl *w0, dfl *w1, dfl *w2, const float *eps, const double *e, const bool *use,
                   cudaStream_t s) {
  const int u = (use[0] ? 1 : 0) | (use[1] ? 2 : 0) | (use[2] ? 4 : 0);
  count_launch(fld<double>(g, 3) + fld<float>(g, 1));
  k_rf_eps_face_e<<<nblk(g.nreal()), TPB, 0, s>>>(g, reinterpret_cast<float2 *>(w0), reinterpret_cast<float2 *>(w1),
                                                  reinterpret_cast<float2 *>(w2), eps, dfl::from_double(e[0]),
                                                  dfl::from_double(e[1]), dfl::from_double(e[2]), u);
}
// fields the fused divergence pass reads and writes: the used components,
// the base (when given) and the output
static double mode_fields(int use_bits, const dfl *base) {
  return (double)(((use_bits >> 0) & 1) + ((use_bits >> 1) & 1) + ((use_bits >> 2) & 1)) + (base ? 1.0 : 0.0) + 1.0;
}
void rf_div_combine(const Grid &g, const RefineTables &t, const dfl *w0, const dfl *w1, const dfl *w2,
                    const bool *use, const dfl *base, dfl *out, int mode, float prescale, bool acc64,
                    double *partials, double *scal, int slot, cudaStream_t s, const float *prescale_dev) {
  const int u = (use[0] ? 1 : 0) | (use[1] ? 2 : 0) | (use[2] ? 4 : 0);
  const float4 *a0 = reinterpret_cast<const float4 *>(w0), *a1 = reinterpret_cast<const float4 *>(w1),
               *a2 = reinterpret_cast<const float4 *>(w2);
  const float4 *b = reinterpret_cast<const float4 *>(base);
  float4 *o = reinterpret_cast<float4 *>(out);
  // post: 1/N, and 1/prescale^2 for the FP32 sums
  const double post = (acc64 ? 1.0 : 1.0 / ((double)prescale * (double)prescale)) / (double)g.nreal();
  count_launch(fld<double>(g, mode_fields(u, base)));
  if (acc64)
    k_rf_div_combine<true>
        <<<DOT_BLOCKS, DOT_TPB, 0, s>>>(g, tab_of(t), a0, a1, a2, u, b, o, mode, prescale, post, partials, nullptr);
  else
    k_rf_div_combine<false><<<DOT_BLOCKS, DOT_TPB, 0, s>>>(g, tab_of(t), a0, a1, a2, u, b, o, mode, prescale, post,
                                                          partials, prescale_dev);
  kdots_finish(partials, DOT_BLOCKS, 1, scal, slot, s);
}

}  // namespace icep
