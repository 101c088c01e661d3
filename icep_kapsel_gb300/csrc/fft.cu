// fft.cu -- batched 3D real FFT kernels (see fft.cuh).
//
// Every 1D transform is a Stockham autosort FFT with radix-8/4/2 stages held
// in registers: a pencil of N complex values is processed by T = N/8 threads,
// each owning one radix-8 (or two radix-4, four radix-2) butterflies per
// stage; stages exchange data through a padded shared-memory tile [N][W+1]
// (W pencils per block, conflict-free). Complex pencils along y and x read
// their first stage straight from global memory and write their last stage
// straight back (coalesced across the W adjacent pencils). The inverse is
// conj(FFT(conj(x))), so only forward kernels and twiddles exist.
#include <math.h>
#include <vector>

#include "fft.cuh"

namespace icep {

namespace {

template <typename R>
__device__ __forceinline__ cplx<R> cadd(cplx<R> a, cplx<R> b) { return cplx<R>{a.x + b.x, a.y + b.y}; }
template <typename R>
__device__ __forceinline__ cplx<R> csub(cplx<R> a, cplx<R> b) { return cplx<R>{a.x - b.x, a.y - b.y}; }
template <typename R>
__device__ __forceinline__ cplx<R> cmul(cplx<R> a, cplx<R> b) {
  return cplx<R>{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename R>
__device__ __forceinline__ cplx<R> mul_mi(cplx<R> a) { return cplx<R>{a.y, -a.x}; }  // * (-i)
template <typename R>
__device__ __forceinline__ cplx<R> conj_if(cplx<R> a, bool c) { return c ? cplx<R>{a.x, -a.y} : a; }

// In-register DFTs, forward kernel exp(-2 pi i nk / r), natural order.
template <typename R>
__device__ __forceinline__ void dft2(cplx<R> *v) {
  const cplx<R> a = v[0];
  v[0] = cadd(a, v[1]);
  v[1] = csub(a, v[1]);
}
template <typename R>
__device__ __forceinline__ void dft4(cplx<R> *v) {
  const cplx<R> a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
  const cplx<R> a2 = cadd(v[1], v[3]), a3 = mul_mi(csub(v[1], v[3]));
  v[0] = cadd(a0, a2);
  v[2] = csub(a0, a2);
  v[1] = cadd(a1, a3);
  v[3] = csub(a1, a3);
}
template <typename R>
__device__ __forceinline__ void dft8(cplx<R> *v) {
  cplx<R> e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
  dft4(e);
  dft4(o);
  const R h = (R)0.70710678118654752440084436210484903928;
  // W8^1 = (1 - i)/sqrt2, W8^2 = -i, W8^3 = -(1 + i)/sqrt2
  const cplx<R> t1 = cplx<R>{h * (o[1].x + o[1].y), h * (o[1].y - o[1].x)};
  const cplx<R> t2 = mul_mi(o[2]);
  const cplx<R> t3 = cplx<R>{h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y)};
  v[0] = cadd(e[0], o[0]);
  v[4] = csub(e[0], o[0]);
  v[1] = cadd(e[1], t1);
  v[5] = csub(e[1], t1);
  v[2] = cadd(e[2], t2);
  v[6] = csub(e[2], t2);
  v[3] = cadd(e[3], t3);
  v[7] = csub(e[3], t3);
}
template <typename R, int RAD>
__device__ __forceinline__ void dftr(cplx<R> *v) {
  if (RAD == 8) dft8(v);
  else if (RAD == 4) dft4(v);
  else dft2(v);
}

// Radix of stage s for a length-N transform: radix-8 stages first, then the
// remainder (N = 8: 8; 16: 8,2; 32: 8,4; 64: 8,8; 128: 8,8,2; 256: 8,8,4).
template <int N>
struct Plan {
  static constexpr int nstages = (N == 8) ? 1 : (N <= 64) ? 2 : 3;
  __host__ __device__ static constexpr int radix(int s) {
    return (N == 8) ? 8
         : (N == 16) ? (s == 0 ? 8 : 2)
         : (N == 32) ? (s == 0 ? 8 : 4)
         : (N == 64) ? 8
         : (N == 128) ? (s < 2 ? 8 : 2)
         : (s < 2 ? 8 : 4);
  }
};

// A global pencil: element e at data[base + e*stride].
template <typename R>
struct GPencil {
  cplx<R> *data;
  long base;
  long stride;
  bool valid;
};

// One Stockham stage of radix RAD on pencil w. Ls: product of the previous
// radices. Input index jb + q*N/RAD, twiddle exp(-2 pi i p q/(Ls RAD)),
// output index k*Ls*RAD + p + Ls*q (jb = k*Ls + p).
// mode bit 0: read from global (first stage), bit 1: write to global (last).
template <typename R, int N, int RAD>
__device__ __forceinline__ void stage(const cplx<R> *__restrict__ src, cplx<R> *__restrict__ dst, int sw, int w, int tid,
                                      int Ls, const cplx<R> *__restrict__ tws, const GPencil<R> &gp, int mode,
                                      bool conj_in, bool conj_out) {
  constexpr int T = N / 8;
  constexpr int NB = 8 / RAD;  // butterflies per thread
#pragma unroll
  for (int m = 0; m < NB; m++) {
    const int jb = tid + T * m;
    const int p = jb & (Ls - 1);
    const int k = jb / Ls;
    cplx<R> v[RAD];
#pragma unroll
    for (int q = 0; q < RAD; q++) {
      const int e = jb + q * (N / RAD);
      cplx<R> x;
      if (mode & 1) x = gp.valid ? gp.data[gp.base + e * gp.stride] : cplx<R>{0, 0};
      else x = src[e * sw + w];
      v[q] = conj_if(x, conj_in);
    }
    if (Ls > 1) {
      const int step = N / (Ls * RAD);
#pragma unroll
      for (int q = 1; q < RAD; q++) v[q] = cmul(v[q], tws[(p * q * step) & (N - 1)]);
    }
    dftr<R, RAD>(v);
#pragma unroll
    for (int q = 0; q < RAD; q++) {
      const int o = k * Ls * RAD + p + Ls * q;
      const cplx<R> y = conj_if(v[q], conj_out);
      if (mode & 2) {
        if (gp.valid) gp.data[gp.base + o * gp.stride] = y;
      } else {
        dst[o * sw + w] = y;
      }
    }
  }
}

// Full length-N transform of pencil w (every thread of the block calls it).
// in_global/out_global select the first stage's source and the last stage's
// sink; tiles a/b alternate. Returns the tile holding the result when the
// last stage does not write to global memory.
template <typename R, int N>
__device__ cplx<R> *pencil_fft(cplx<R> *a, cplx<R> *b, int sw, int w, int tid, const cplx<R> *tws,
                               const GPencil<R> &gp, bool in_global, bool out_global, bool inverse) {
  cplx<R> *src = a, *dst = b;
  int Ls = 1;
#pragma unroll
  for (int s = 0; s < Plan<N>::nstages; s++) {
    constexpr int dummy = 0;
    (void)dummy;
    const int rad = Plan<N>::radix(s);
    const bool first = (s == 0), last = (s == Plan<N>::nstages - 1);
    const int mode = (first && in_global ? 1 : 0) | (last && out_global ? 2 : 0);
    const bool ci = first && inverse, co = last && inverse;
    if (rad == 8) stage<R, N, 8>(src, dst, sw, w, tid, Ls, tws, gp, mode, ci, co);
    else if (rad == 4) stage<R, N, 4>(src, dst, sw, w, tid, Ls, tws, gp, mode, ci, co);
    else stage<R, N, 2>(src, dst, sw, w, tid, Ls, tws, gp, mode, ci, co);
    Ls *= rad;
    if (!(last && out_global)) {
      __syncthreads();
      cplx<R> *t = src;
      src = dst;
      dst = t;
    }
  }
  return src;
}

template <typename R>
__device__ __forceinline__ void load_twiddles(cplx<R> *tws, const cplx<R> *__restrict__ tw, int n) {
  const int lin = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  for (int q = lin; q < n; q += nthr) tws[q] = tw[q];
}

// Complex FFT along y (axis 1) or x (axis 0); W pencils per block, blockDim (W, N/8).
template <typename R, int N>
__global__ void __launch_bounds__(1024) k_pencils(FieldBatch<R> fb, Grid g, int axis, int W, int tiles_per_row,
                                                  const cplx<R> *__restrict__ tw, int inverse) {
  extern __shared__ unsigned char smem_raw[];
  const int sw = W + 1;
  cplx<R> *tws = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *ta = tws + N;
  cplx<R> *tb = ta + N * sw;
  GPencil<R> gp;
  gp.data = reinterpret_cast<cplx<R> *>(fb.p[blockIdx.y]);
  const int w = threadIdx.x, tid = threadIdx.y;
  if (axis == 1) {
    const int i = blockIdx.x / tiles_per_row;
    const int kz = (blockIdx.x % tiles_per_row) * W + w;
    gp.valid = kz < g.hnz;
    gp.base = (long)i * g.ny * g.hnz + kz;
    gp.stride = g.hnz;
  } else {
    const long q = (long)blockIdx.x * W + w;
    gp.valid = q < (long)g.ny * g.hnz;
    gp.base = q;
    gp.stride = (long)g.ny * g.hnz;
  }
  load_twiddles(tws, tw, N);
  __syncthreads();
  pencil_fft<R, N>(ta, tb, sw, w, tid, tws, gp, true, true, inverse != 0);
}

// z rows, forward: NZ reals -> NZ/2+1 complex through an H = NZ/2-point
// complex FFT of z[m] = x[2m] + i x[2m+1] and X[k] = E[k] + exp(-2 pi i k/NZ) O[k].
template <typename R, int H>
__global__ void __launch_bounds__(1024) k_rows_r2c(FieldBatch<R> fb, Grid g, int W, const cplx<R> *__restrict__ tw,
                                                   const cplx<R> *__restrict__ post) {
  extern __shared__ unsigned char smem_raw[];
  const int sw = W + 1;
  cplx<R> *tws = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *ta = tws + H;
  cplx<R> *tb = ta + H * sw;
  R *data = fb.p[blockIdx.y];
  const long nrows = (long)g.nx * g.ny;
  const long row0 = (long)blockIdx.x * W;
  const int nthr = blockDim.x * blockDim.y;
  const int lin = threadIdx.y * blockDim.x + threadIdx.x;
  load_twiddles(tws, tw, H);
  for (int q = lin; q < W * H; q += nthr) {  // row-major, coalesced
    const int w = q / H, e = q - w * H;
    const long row = row0 + w;
    cplx<R> v{0, 0};
    if (row < nrows) {
      const R *rp = data + row * g.nzp;
      v.x = rp[2 * e];
      v.y = rp[2 * e + 1];
    }
    ta[e * sw + w] = v;
  }
  __syncthreads();
  GPencil<R> gp{nullptr, 0, 0, false};
  cplx<R> *Z = pencil_fft<R, H>(ta, tb, sw, threadIdx.x, threadIdx.y, tws, gp, false, false, false);
  for (int q = lin; q < W * (H + 1); q += nthr) {
    const int wr = q / (H + 1), k = q - wr * (H + 1);
    const long row = row0 + wr;
    if (row >= nrows) continue;
    const int k1 = (k == H) ? 0 : k, k2 = (k == 0) ? 0 : H - k;
    const cplx<R> z = Z[k1 * sw + wr];
    cplx<R> c = Z[k2 * sw + wr];
    c.y = -c.y;
    const R er = R(0.5) * (z.x + c.x), ei = R(0.5) * (z.y + c.y);
    const R orr = R(0.5) * (z.y - c.y), oi = R(-0.5) * (z.x - c.x);
    const cplx<R> pw = post[k];
    R *rp = data + row * g.nzp;
    rp[2 * k] = er + (pw.x * orr - pw.y * oi);
    rp[2 * k + 1] = ei + (pw.x * oi + pw.y * orr);
  }
}

// z rows, inverse: half spectrum -> NZ reals, scaled; the imaginary parts of
// kz = 0 and kz = NZ/2 are ignored (as in a standard real inverse).
template <typename R, int H>
__global__ void __launch_bounds__(1024) k_rows_c2r(FieldBatch<R> fb, Grid g, int W, const cplx<R> *__restrict__ tw,
                                                   const cplx<R> *__restrict__ post, R scale) {
  extern __shared__ unsigned char smem_raw[];
  const int sw = W + 1;
  cplx<R> *tws = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *ta = tws + H;
  cplx<R> *tb = ta + H * sw;
  cplx<R> *sx = tb + H * sw;  // staged half spectrum, rows of H+1 (+1 pad)
  const int sxw = H + 2;
  R *data = fb.p[blockIdx.y];
  const long nrows = (long)g.nx * g.ny;
  const long row0 = (long)blockIdx.x * W;
  const int nthr = blockDim.x * blockDim.y;
  const int lin = threadIdx.y * blockDim.x + threadIdx.x;
  load_twiddles(tws, tw, H);
  for (int q = lin; q < W * (H + 1); q += nthr) {
    const int w = q / (H + 1), k = q - w * (H + 1);
    const long row = row0 + w;
    cplx<R> v{0, 0};
    if (row < nrows) {
      const R *rp = data + row * g.nzp;
      v.x = rp[2 * k];
      v.y = (k == 0 || k == H) ? R(0) : rp[2 * k + 1];
    }
    sx[w * sxw + k] = v;
  }
  __syncthreads();
  for (int q = lin; q < W * H; q += nthr) {
    const int w = q / H, k = q - w * H;
    const cplx<R> x = sx[w * sxw + k];
    cplx<R> c = sx[w * sxw + (H - k)];
    c.y = -c.y;
    const R sr = x.x + c.x, si = x.y + c.y;
    const R dr = x.x - c.x, di = x.y - c.y;
    const cplx<R> pw = post[k];  // exp(-2 pi i k/NZ); use its conjugate
    const R wr = pw.x, wi = -pw.y;
    const R tr = wr * dr - wi * di, ti = wr * di + wi * dr;
    ta[k * sw + w] = cplx<R>{sr - ti, si + tr};
  }
  __syncthreads();
  GPencil<R> gp{nullptr, 0, 0, false};
  cplx<R> *z = pencil_fft<R, H>(ta, tb, sw, threadIdx.x, threadIdx.y, tws, gp, false, false, true);
  for (int q = lin; q < W * H; q += nthr) {
    const int wr = q / H, m = q - wr * H;
    const long row = row0 + wr;
    if (row >= nrows) continue;
    R *rp = data + row * g.nzp;
    const cplx<R> v = z[m * sw + wr];
    rp[2 * m] = v.x * scale;
    rp[2 * m + 1] = v.y * scale;
    if (m == 0) {  // padding of a real-space row
      rp[g.nz] = R(0);
      rp[g.nz + 1] = R(0);
    }
  }
}

// Hermitian completion of the kz = 0 and kz = NZ/2 planes with the kept
// halves of the reference's inverse (rdft3dsort, fftsg3d.c:645-667):
// kz = 0 keeps 1 <= j <= NY/2-1 and (j in {0,NY/2}, i <= NX/2); kz = NZ/2
// keeps the complement; self-conjugate points keep their real part.
// Dropped entries read their (kept) mirror, kept entries are only written at
// self-conjugate points, so the update is race-free in place.
template <typename R>
__global__ void k_herm_project(FieldBatch<R> fb, Grid g) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long plane = (long)g.nx * g.ny;
  if (t >= 2 * plane) return;
  const int pz = (int)(t / plane);
  const long ij = t - pz * plane;
  const int i = (int)(ij / g.ny), j = (int)(ij - (long)i * g.ny);
  const int kz = pz ? g.nz / 2 : 0;
  const int mi = (g.nx - i) % g.nx, mj = (g.ny - j) % g.ny;
  bool kept;
  if (j >= 1 && j <= g.ny / 2 - 1) kept = true;
  else if (j == 0 || j == g.ny / 2) kept = (i <= g.nx / 2);
  else kept = false;
  if (pz) kept = !kept;
  R *data = fb.p[blockIdx.y];
  const long at = gidx(g, i, j, 2 * kz);
  if (mi == i && mj == j) {
    data[at + 1] = R(0);
  } else if (!kept) {
    const long m = gidx(g, mi, mj, 2 * kz);
    data[at] = data[m];
    data[at + 1] = -data[m + 1];
  }
}

template <typename R>
constexpr int pencil_width() {
  return (sizeof(R) == 8) ? 8 : 16;
}

// Twiddle table exp(-2 pi i m / denom), m < n. Uploaded on the caller's
// stream and waited for: a pageable-memory copy may still be in flight when
// cudaMemcpy returns, and the library's non-blocking streams do not order
// against the legacy stream.
template <typename R>
cplx<R> *upload_table(int n, int denom, cudaStream_t s) {
  std::vector<cplx<R>> h(n);
  for (int m = 0; m < n; m++) {
    long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)m / (long double)denom;
    h[m].x = (R)cosl(a);
    h[m].y = (R)sinl(a);
  }
  cplx<R> *d = nullptr;
  if (cudaMalloc(&d, sizeof(cplx<R>) * (n > 0 ? n : 1)) != cudaSuccess) return nullptr;
  if (cudaMemcpyAsync(d, h.data(), sizeof(cplx<R>) * n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaFree(d);
    return nullptr;
  }
  return d;
}

// ---- launch helpers (template dispatch on the transform length) ---------
template <typename R>
size_t pencil_smem(int n) {
  const int W = pencil_width<R>();
  return ((size_t)n + 2 * (size_t)n * (W + 1)) * sizeof(cplx<R>);
}
template <typename R>
constexpr int row_width() {
  return 2 * pencil_width<R>();
}
template <typename R>
size_t row_smem(int h, bool inverse) {
  const int W = row_width<R>();
  size_t s = ((size_t)h + 2 * (size_t)h * (W + 1)) * sizeof(cplx<R>);
  if (inverse) s += (size_t)W * (h + 2) * sizeof(cplx<R>);
  return s;
}

template <typename R, int N>
void launch_pencils_n(const FFTPlan<R> &p, const FieldBatch<R> &fb, int axis, bool inverse, cudaStream_t s) {
  const Grid &g = p.g;
  constexpr int W = pencil_width<R>();
  const int tiles_per_row = (g.hnz + W - 1) / W;
  const unsigned nblk = axis == 1 ? (unsigned)(g.nx * tiles_per_row) : div_up((long)g.ny * g.hnz, W);
  count_launch();
  k_pencils<R, N><<<dim3(nblk, fb.n), dim3(W, N / 8), pencil_smem<R>(N), s>>>(
      fb, g, axis, W, tiles_per_row, axis == 0 ? p.tw_x : p.tw_y, inverse ? 1 : 0);
}

template <typename R>
void launch_pencils(const FFTPlan<R> &p, const FieldBatch<R> &fb, int axis, bool inverse, cudaStream_t s) {
  switch (axis == 0 ? p.g.nx : p.g.ny) {
    case 16: launch_pencils_n<R, 16>(p, fb, axis, inverse, s); break;
    case 32: launch_pencils_n<R, 32>(p, fb, axis, inverse, s); break;
    case 64: launch_pencils_n<R, 64>(p, fb, axis, inverse, s); break;
    case 128: launch_pencils_n<R, 128>(p, fb, axis, inverse, s); break;
    default: launch_pencils_n<R, 256>(p, fb, axis, inverse, s); break;
  }
}

template <typename R, int H>
void launch_rows_n(const FFTPlan<R> &p, const FieldBatch<R> &fb, bool inverse, cudaStream_t s) {
  const Grid &g = p.g;
  constexpr int W = row_width<R>();
  const dim3 grid(div_up((long)g.nx * g.ny, W), fb.n);
  const dim3 block(W, H / 8);
  count_launch();
  if (!inverse) {
    k_rows_r2c<R, H><<<grid, block, row_smem<R>(H, false), s>>>(fb, g, W, p.tw_z, p.tw_post);
  } else {
    const R scale = (R)(1.0 / ((double)g.nx * g.ny * g.nz));
    k_rows_c2r<R, H><<<grid, block, row_smem<R>(H, true), s>>>(fb, g, W, p.tw_z, p.tw_post, scale);
  }
}

template <typename R>
void launch_rows(const FFTPlan<R> &p, const FieldBatch<R> &fb, bool inverse, cudaStream_t s) {
  switch (p.g.nz / 2) {
    case 8: launch_rows_n<R, 8>(p, fb, inverse, s); break;
    case 16: launch_rows_n<R, 16>(p, fb, inverse, s); break;
    case 32: launch_rows_n<R, 32>(p, fb, inverse, s); break;
    case 64: launch_rows_n<R, 64>(p, fb, inverse, s); break;
    default: launch_rows_n<R, 128>(p, fb, inverse, s); break;
  }
}

template <typename R>
void launch_herm(const FFTPlan<R> &p, const FieldBatch<R> &fb, cudaStream_t s) {
  const long n = 2L * p.g.nx * p.g.ny;
  count_launch();
  k_herm_project<R><<<dim3(div_up(n, 256), fb.n), 256, 0, s>>>(fb, p.g);
}

template <typename R, int N>
void set_pencil_attr() {
  cudaFuncSetAttribute(k_pencils<R, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pencil_smem<R>(N));
}
template <typename R, int H>
void set_row_attr() {
  cudaFuncSetAttribute(k_rows_r2c<R, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)row_smem<R>(H, false));
  cudaFuncSetAttribute(k_rows_c2r<R, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)row_smem<R>(H, true));
}

}  // namespace

template <typename R>
int fft_plan_init(FFTPlan<R> &p, const Grid &g, cudaStream_t s) {
  p.g = g;
  p.tw_x = upload_table<R>(g.nx, g.nx, s);
  p.tw_y = upload_table<R>(g.ny, g.ny, s);
  p.tw_z = upload_table<R>(g.nz / 2, g.nz / 2, s);
  p.tw_post = upload_table<R>(g.nz / 2 + 1, g.nz, s);
  if (!p.tw_x || !p.tw_y || !p.tw_z || !p.tw_post) return ICEP_ERR_CUDA;
  set_pencil_attr<R, 16>();
  set_pencil_attr<R, 32>();
  set_pencil_attr<R, 64>();
  set_pencil_attr<R, 128>();
  set_pencil_attr<R, 256>();
  set_row_attr<R, 8>();
  set_row_attr<R, 16>();
  set_row_attr<R, 32>();
  set_row_attr<R, 64>();
  set_row_attr<R, 128>();
  return (cudaGetLastError() == cudaSuccess) ? ICEP_OK : ICEP_ERR_CUDA;
}

template <typename R>
void fft_plan_free(FFTPlan<R> &p) {
  cudaFree(p.tw_x);
  cudaFree(p.tw_y);
  cudaFree(p.tw_z);
  cudaFree(p.tw_post);
  p.tw_x = p.tw_y = p.tw_z = p.tw_post = nullptr;
}

template <typename R>
void fft_r2c(const FFTPlan<R> &p, const FieldBatch<R> &fb, cudaStream_t s) {
  launch_rows(p, fb, false, s);
  launch_pencils(p, fb, 1, false, s);
  launch_pencils(p, fb, 0, false, s);
}

template <typename R>
void fft_c2r(const FFTPlan<R> &p, const FieldBatch<R> &fb, cudaStream_t s) {
  launch_herm(p, fb, s);
  launch_pencils(p, fb, 0, true, s);
  launch_pencils(p, fb, 1, true, s);
  launch_rows(p, fb, true, s);
}

template <typename R>
void fft_pass(const FFTPlan<R> &p, const FieldBatch<R> &fb, int pass, cudaStream_t s) {
  switch (pass) {
    case 0: launch_rows(p, fb, false, s); break;
    case 1: launch_pencils(p, fb, 1, false, s); break;
    case 2: launch_pencils(p, fb, 0, false, s); break;
    case 3: launch_herm(p, fb, s); break;
    case 4: launch_pencils(p, fb, 0, true, s); break;
    case 5: launch_pencils(p, fb, 1, true, s); break;
    default: launch_rows(p, fb, true, s); break;
  }
}

template void fft_pass<double>(const FFTPlan<double> &, const FieldBatch<double> &, int, cudaStream_t);
template void fft_pass<float>(const FFTPlan<float> &, const FieldBatch<float> &, int, cudaStream_t);
template int fft_plan_init<double>(FFTPlan<double> &, const Grid &, cudaStream_t);
template int fft_plan_init<float>(FFTPlan<float> &, const Grid &, cudaStream_t);
template void fft_plan_free<double>(FFTPlan<double> &);
template void fft_plan_free<float>(FFTPlan<float> &);
template void fft_r2c<double>(const FFTPlan<double> &, const FieldBatch<double> &, cudaStream_t);
template void fft_r2c<float>(const FFTPlan<float> &, const FieldBatch<float> &, cudaStream_t);
template void fft_c2r<double>(const FFTPlan<double> &, const FieldBatch<double> &, cudaStream_t);
template void fft_c2r<float>(const FFTPlan<float> &, const FieldBatch<float> &, cudaStream_t);

}  // namespace icep
