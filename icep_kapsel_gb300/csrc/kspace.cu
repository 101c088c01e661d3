// kspace.cu -- see kspace.cuh.
#include "krylov.cuh"
#include "kspace.cuh"

namespace icep {

namespace {

constexpr int TPB = 256;

struct KMode {
  int i, j, kz;
  long im;
};

__device__ __forceinline__ bool kmode(const Grid &g, unsigned t, KMode &m) {
  if (t >= (unsigned)g.nmodes()) return false;
  mode_ijk3(g, t, m.i, m.j, m.kz);
  m.im = gidx(g, m.i, m.j, 2 * m.kz);
  return true;
}

__device__ __forceinline__ int kweight(const Grid &g, const KMode &m) { return read_weight(g, m.i, m.j, m.kz); }

// Value of vector a at a read mode (weight > 0) as the inverse transform
// sees it: the stored entry, real part only at self-conjugate points.
template <typename R>
__device__ __forceinline__ void ld(const R *__restrict__ a, const KMode &m, int w, R &re, R &im) {
  re = a[m.im];
  im = (w == 1) ? R(0) : a[m.im + 1];
}

struct R2 {
  float x, y;
};
__device__ __forceinline__ void ldv(const float *a, const KMode &m, int wt, R2 &v) {
  v.x = a[m.im];
  v.y = (wt == 1) ? 0.f : a[m.im + 1];
}

template <typename R>
__device__ __forceinline__ void kvec(const Grid &g, const KMode &m, R *k) {
  k[0] = wave_of<R>(g, 0) * (R)kx_of(g, m.i);
  k[1] = wave_of<R>(g, 1) * (R)ky_of(g, m.j);
  k[2] = wave_of<R>(g, 2) * (R)m.kz;
}


#define KTID ((unsigned)(blockIdx.x * blockDim.x + threadIdx.x))

template <typename R>
__global__ void k_kdots(Grid g, const R *a0, const R *b0, const R *a1, const R *b1, int n, double *partials) {
  // the thread's terms in the field type (FP32 in MIXED precision: FP64 is
  // scarce on GB300), the block and grid sums in FP64
  R s0 = R(0), s1 = R(0);
  const unsigned N = (unsigned)g.nmodes();
  for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < N; t += gridDim.x * blockDim.x) {
    KMode m;
    kmode(g, t, m);
    const int w = kweight(g, m);
    if (w == 0) continue;
    R ar, ai, br, bi;
    ld(a0, m, w, ar, ai);
    ld(b0, m, w, br, bi);
    s0 += (R)w * (ar * br + ai * bi);
    if (n > 1) {
      ld(a1, m, w, ar, ai);
      ld(b1, m, w, br, bi);
      s1 += (R)w * (ar * br + ai * bi);
    }
  }
  // warp sums in the field type, one FP64 value per warp
  __shared__ double red[2][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
  }
  if (lane == 0) {
    red[0][wid] = (double)s0;
    red[1][wid] = (double)s1;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += red[threadIdx.x][w];
    partials[blockIdx.x * 2 + threadIdx.x] = v * (1.0 / (double)g.nreal());
  }
}

__global__ void k_kdots_final(const double *partials, int nblocks, int n, double *scal, int slot) {
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

// The vector updates touch read modes only; each thread reads and writes its
// own mode, so the updates may run in place.
template <typename R>
__global__ void k_kbicg_p(Grid g, R *p, const R *r, const R *v, R beta, R w) {
  KMode m;
  if (!kmode(g, KTID, m)) return;
  const int wt = kweight(g, m);
  if (wt == 0) return;
  R rr, ri, pr, pi, vr, vi;
  ld(r, m, wt, rr, ri);
  ld(p, m, wt, pr, pi);
  ld(v, m, wt, vr, vi);
  p[m.im] = rr + beta * (pr - w * vr);
  p[m.im + 1] = ri + beta * (pi - w * vi);
}

template <typename R>
__global__ void k_kbicg_s(Grid g, R *sv, const R *r, const R *v, double rho, const double *scal) {
  KMode m;
  if (!kmode(g, KTID, m)) return;
  const int wt = kweight(g, m);
  if (wt == 0) return;
  const R alpha = (R)(rho / scal[S_R0V]);
  R rr, ri, vr, vi;
  ld(r, m, wt, rr, ri);
  ld(v, m, wt, vr, vi);
  sv[m.im] = rr - alpha * vr;
  sv[m.im + 1] = ri - alpha * vi;
}

template <typename R>
__global__ void k_kbicg_xr(Grid g, R *xt, R *r, const R *p, const R *sv, const R *t, double rho, const double *scal) {
  KMode m;
  if (!kmode(g, KTID, m)) return;
  const int wt = kweight(g, m);
  if (wt == 0) return;
  const R alpha = (R)(rho / scal[S_R0V]);
  const double tt = scal[S_TT];
  const R w = (R)((tt > 0.0) ? scal[S_TS] / tt : 0.0);
  R pr, pi, sr, si, tr, ti, xr, xi;
  ld(p, m, wt, pr, pi);
  ld(sv, m, wt, sr, si);
  ld(t, m, wt, tr, ti);
  ld(xt, m, wt, xr, xi);
  xt[m.im] = xr + alpha * pr + w * sr;
  xt[m.im + 1] = xi + alpha * pi + w * si;
  r[m.im] = sr - w * tr;
  r[m.im + 1] = si - w * ti;
}

template <typename R>
__device__ __forceinline__ R kmult(const R *k, R ieps) {
  const R k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
  return (k2 > R(0)) ? -ieps / k2 : R(0);
}

template <typename R>
__global__ void k_kgrad_pre(Grid g, const R *p, R *g0, R *g1, R *g2, R ieps) {
  KMode m;
  if (!kmode(g, KTID, m)) return;
  const int wt = kweight(g, m);
  if (wt == 0) return;
  R k[3];
  kvec(g, m, k);
  const R mm = kmult(k, ieps);
  R re, im;
  ld(p, m, wt, re, im);
  re *= mm;
  im *= mm;
  const int idx[3] = {m.i, m.j, m.kz};
  R *out[3] = {g0, g1, g2};
#pragma unroll
  for (int c = 0; c < 3; c++) {
    // i k_c (re + i im) = (-k_c im, k_c re), then * exp(i dx k_c / 2)
    const R gr = -k[c] * im, gi = k[c] * re;
    R sn, cs;
    shift_of(g, c, idx[c], cs, sn);
    out[c][m.im] = gr * cs - gi * sn;
    out[c][m.im + 1] = gr * sn + gi * cs;
  }
}

template <typename R>
__global__ void k_kdiv_post(Grid g, const R *w0, const R *w1, const R *w2, R *v) {
  KMode m;
  if (!kmode(g, KTID, m)) return;
  if (kweight(g, m) == 0) return;
  R k[3];
  kvec(g, m, k);
  const int idx[3] = {m.i, m.j, m.kz};
  const R *w[3] = {w0, w1, w2};
  R sr = R(0), si = R(0);
#pragma unroll
  for (int c = 0; c < 3; c++) {
    R sn, cs;
    shift_of(g, c, idx[c], cs, sn);
    const R ksr = k[c] * cs, ksi = -k[c] * sn;  // k_c conj(s_c)
    const R ur = w[c][m.im], ui = w[c][m.im + 1];
    sr += ur * ksr - ui * ksi;
    si += ur * ksi + ui * ksr;
  }
  v[m.im] = -si;  // i (sr + i si)
  v[m.im + 1] = sr;
}

// ieps_dev (if given: 1/eps_ref as a device double) replaces ieps
template <typename R>
__global__ void k_kprecond(Grid g, const R *x, R *y, R ieps, const double *ieps_dev) {
  KMode m;
  if (!kmode(g, KTID, m)) return;
  if (ieps_dev) ieps = (R)*ieps_dev;
  const int wt = kweight(g, m);
  if (wt == 0) return;
  R k[3];
  kvec(g, m, k);
  const R mm = kmult(k, ieps);
  R re, im;
  ld(x, m, wt, re, im);
  y[m.im] = mm * re;
  y[m.im + 1] = mm * im;
}

// groups of four vectors per pass keep the accumulators in registers
__global__ void k_kmdot(Grid g, KVecs V, int nv, const float *w, double *partials) {
  __shared__ double red[4][32];
  const unsigned N = (unsigned)g.nmodes();
  const double inv = 1.0 / (double)g.nreal();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int i0 = 0; i0 < nv; i0 += 4) {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < N; t += gridDim.x * blockDim.x) {
      KMode m;
      kmode(g, t, m);
      const int wt = kweight(g, m);
      if (wt == 0) continue;
      R2 wv;
      ldv(w, m, wt, wv);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (i0 + q < nv) {
          R2 a;
          ldv(V.p[i0 + q], m, wt, a);
          acc[q] += (double)wt * ((double)a.x * (double)wv.x + (double)a.y * (double)wv.y);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      double v = acc[q] * inv;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) red[q][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4 && i0 + (int)threadIdx.x < nv) {
      double t2 = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); q++) t2 += red[threadIdx.x][q];
      partials[(long)blockIdx.x * nv + i0 + threadIdx.x] = t2;
    }
    __syncthreads();
  }
}

__global__ void k_kmdot_final(const double *partials, int nblocks, int nv, double *out) {
  const int i = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partials[(long)b * nv + i];
  __shared__ double red[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) red[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t2 = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) t2 += red[q];
    out[i] = t2;
  }
}

__global__ void k_kmaxpy(Grid g, float *w, KVecs V, int nv, const double *coef, float sign) {
  KMode m;
  if (!kmode(g, KTID, m)) return;
  const int wt = kweight(g, m);
  if (wt == 0) return;
  R2 a;
  ldv(w, m, wt, a);
  for (int i = 0; i < nv; i++) {
    R2 v;
    ldv(V.p[i], m, wt, v);
    const float c = sign * (float)coef[i];
    a.x += c * v.x;
    a.y += c * v.y;
  }
  w[m.im] = a.x;
  w[m.im + 1] = a.y;
}

__global__ void k_kscale_by_norm(Grid g, const float *w, float *out, const double *nrm2) {
  KMode m;
  if (!kmode(g, KTID, m)) return;
  const int wt = kweight(g, m);
  if (wt == 0) return;
  const double n2 = *nrm2;
  const float f = (n2 > 0.0) ? (float)(1.0 / sqrt(n2)) : 0.f;
  R2 a;
  ldv(w, m, wt, a);
  out[m.im] = f * a.x;
  out[m.im + 1] = f * a.y;
}

__global__ void k_kadd(Grid g, const float *v, const float *z, float *xt) {
  KMode m;
  if (!kmode(g, KTID, m)) return;
  const int wt = kweight(g, m);
  if (wt == 0) return;
  R2 a, b;
  ldv(v, m, wt, a);
  ldv(z, m, wt, b);
  xt[m.im] = a.x + b.x;
  xt[m.im + 1] = a.y + b.y;
}

__global__ void k_ksub(Grid g, const float *b, const float *w, float *r) {
  KMode m;
  if (!kmode(g, KTID, m)) return;
  const int wt = kweight(g, m);
  if (wt == 0) return;
  R2 x, y;
  ldv(b, m, wt, x);
  ldv(w, m, wt, y);
  r[m.im] = x.x - y.x;
  r[m.im + 1] = x.y - y.y;
}

inline unsigned nblk(const Grid &g) { return div_up(g.nmodes(), TPB); }

}  // namespace

void kdots_finish(const double *partials, int nblocks, int n, double *scal, int slot, cudaStream_t s) {
  count_launch();
  k_kdots_final<<<1, 256, 0, s>>>(partials, nblocks, n, scal, slot);
}

template <typename R>
void kdots(const Grid &g, const R *a0, const R *b0, const R *a1, const R *b1, int n, double *partials, double *scal,
           int slot, cudaStream_t s) {
  count_launch(fld<R>(g, ndistinct(a0, b0, n > 1 ? a1 : nullptr, n > 1 ? b1 : nullptr)));
  k_kdots<R><<<DOT_BLOCKS, DOT_TPB, 0, s>>>(g, a0, b0, a1, b1, n, partials);
  count_launch();
  k_kdots_final<<<1, 256, 0, s>>>(partials, DOT_BLOCKS, n, scal, slot);
}
template <typename R>
void kbicg_p(const Grid &g, R *p, const R *r, const R *v, double beta, double w, cudaStream_t s) {
  count_launch(fld<R>(g, 4));
  k_kbicg_p<R><<<nblk(g), TPB, 0, s>>>(g, p, r, v, (R)beta, (R)w);
}
template <typename R>
void kbicg_s(const Grid &g, R *sv, const R *r, const R *v, double rho, const double *scal, cudaStream_t s) {
  count_launch(fld<R>(g, 3));
  k_kbicg_s<R><<<nblk(g), TPB, 0, s>>>(g, sv, r, v, rho, scal);
}
template <typename R>
void kbicg_xr(const Grid &g, R *xt, R *r, const R *p, const R *sv, const R *t, double rho, const double *scal,
              cudaStream_t s) {
  count_launch(fld<R>(g, 6));
  k_kbicg_xr<R><<<nblk(g), TPB, 0, s>>>(g, xt, r, p, sv, t, rho, scal);
}
template <typename R>
void kgrad_pre(const Grid &g, const R *p, R *g0, R *g1, R *g2, double eps_ref, cudaStream_t s) {
  count_launch(fld<R>(g, 4));
  k_kgrad_pre<R><<<nblk(g), TPB, 0, s>>>(g, p, g0, g1, g2, (R)(1.0 / eps_ref));
}
template <typename R>
void kdiv_post(const Grid &g, const R *w0, const R *w1, const R *w2, R *v, cudaStream_t s) {
  count_launch(fld<R>(g, 4));
  k_kdiv_post<R><<<nblk(g), TPB, 0, s>>>(g, w0, w1, w2, v);
}
template <typename R>
void kprecond(const Grid &g, const R *x, R *y, double eps_ref, cudaStream_t s) {
  count_launch(fld<R>(g, 2));
  k_kprecond<R><<<nblk(g), TPB, 0, s>>>(g, x, y, (R)(1.0 / eps_ref), nullptr);
}
template <typename R>
void kprecond(const Grid &g, const R *x, R *y, const double *ieps_dev, cudaStream_t s) {
  count_launch(fld<R>(g, 2));
  k_kprecond<R><<<nblk(g), TPB, 0, s>>>(g, x, y, R(0), ieps_dev);
}

void kmdot(const Grid &g, const KVecs &V, int nv, const float *w, double *partials, cudaStream_t s) {
  count_launch(fld<float>(g, nv + 1.0));
  k_kmdot<<<DOT_BLOCKS, DOT_TPB, 0, s>>>(g, V, nv, w, partials);
}
void kmdot_final(const double *partials, int nv, double *out, cudaStream_t s) {
  count_launch();
  k_kmdot_final<<<nv, 256, 0, s>>>(partials, DOT_BLOCKS, nv, out);
}
void kmaxpy(const Grid &g, float *w, const KVecs &V, int nv, const double *coef, double sign, cudaStream_t s) {
  count_launch(fld<float>(g, nv + 2.0));
  k_kmaxpy<<<nblk(g), TPB, 0, s>>>(g, w, V, nv, coef, (float)sign);
}
void kscale_by_norm(const Grid &g, const float *w, float *out, const double *nrm2, cudaStream_t s) {
  count_launch(fld<float>(g, 2));
  k_kscale_by_norm<<<nblk(g), TPB, 0, s>>>(g, w, out, nrm2);
}
void kadd(const Grid &g, const float *v, const float *z, float *xt, cudaStream_t s) {
  count_launch(fld<float>(g, 3));
  k_kadd<<<nblk(g), TPB, 0, s>>>(g, v, z, xt);
}
void ksub(const Grid &g, const float *b, const float *w, float *r, cudaStream_t s) {
  count_launch(fld<float>(g, 3));
  k_ksub<<<nblk(g), TPB, 0, s>>>(g, b, w, r);
}

#define KS_INST(R)                                                                                                 \
  template void kdots<R>(const Grid &, const R *, const R *, const R *, const R *, int, double *, double *, int,   \
                         cudaStream_t);                                                                            \
  template void kbicg_p<R>(const Grid &, R *, const R *, const R *, double, double, cudaStream_t);                 \
  template void kbicg_s<R>(const Grid &, R *, const R *, const R *, double, const double *, cudaStream_t);         \
  template void kbicg_xr<R>(const Grid &, R *, R *, const R *, const R *, const R *, double, const double *,       \
                            cudaStream_t);                                                                         \
  template void kgrad_pre<R>(const Grid &, const R *, R *, R *, R *, double, cudaStream_t);                        \
  template void kdiv_post<R>(const Grid &, const R *, const R *, const R *, R *, cudaStream_t);                    \
  template void kprecond<R>(const Grid &, const R *, R *, double, cudaStream_t);                                      \
  template void kprecond<R>(const Grid &, const R *, R *, const double *, cudaStream_t);

KS_INST(double)
KS_INST(float)

}  // namespace icep
