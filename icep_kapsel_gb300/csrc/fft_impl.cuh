// fft_impl.cuh -- batched 3D real FFT kernels and their launchers (see
// fft.cuh), templated on the arithmetic type. Instantiated for float and
// double in fft.cu and for float-float (dfl) in fft_df.cu.
//
// The 1D transforms and the x-plane cores are in fft_blocks.cuh.
//
// A 3D transform is two passes when an x-plane fits in shared memory:
//   forward: plane pass (z rows real->complex, then y pencils) + x pass;
//   inverse: x pass + plane pass (y pencils, then z rows complex->real).
// Larger planes use separate z-row and y-pencil passes. The reference's
// treatment of the kz = 0 and kz = NZ/2 planes in its inverse (Ooura's
// rdft3dsort reads half of each plane, the rest is implied by Hermitian
// symmetry) is reproduced inside the inverse passes: the i-direction part on
// the four special x pencils as they are loaded, the j-direction part on the
// two special columns of each x-plane.
#pragma once
#include <math.h>

#include <type_traits>
#include <vector>

#include "fft.cuh"
#include "fft_blocks.cuh"
#include "kop.cuh"

namespace icep {

namespace {

// ---- plane kernels (one block per x-plane and field) ---------------------
template <typename R, int NY, int H>
__global__ void __launch_bounds__(1024) k_plane_fwd(FieldBatch<R> fb, Grid g, const cplx<R> *__restrict__ twy,
                                                    const cplx<R> *__restrict__ twz, const cplx<R> *__restrict__ post) {
  extern __shared__ unsigned char smem_raw[];
  cplx<R> *sty = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *stz = sty + NY;
  cplx<R> *spost = stz + H;
  cplx<R> *A = spost + (H + 1);
  cplx<R> *B = A + plane_tile(NY, H);
  const int i = blockIdx.x;
  R *data = fb.p[blockIdx.y];
  const int nthr = blockDim.x * blockDim.y, lin = threadIdx.y * blockDim.x + threadIdx.x;
  load_table(sty, twy, NY);
  load_table(stz, twz, H);
  load_table(spost, post, H + 1);
  // rows j of the plane as H-point complex pencils, element-major in A
  const R *plane = data + (long)i * NY * g.nzp;
  constexpr int rsw = NY + 1;
  for (int q = lin; q < NY * H; q += nthr) {
    const int j = q / H, e = q - j * H;
    const R *rp = plane + (long)j * g.nzp;
    A[e * rsw + j] = cplx<R>{rp[2 * e], rp[2 * e + 1]};
  }
  __syncthreads();
  GPencils<R> outp{reinterpret_cast<cplx<R> *>(data), (long)i * NY * g.hnz, 1, g.hnz, H + 1};
  plane_fwd_core<R, NY, H>(A, B, sty, stz, spost, outp);
}

template <typename R, int NY, int H>
__global__ void __launch_bounds__(1024) k_plane_inv(FieldBatch<R> fb, Grid g, const cplx<R> *__restrict__ twy,
                                                    const cplx<R> *__restrict__ twz, const cplx<R> *__restrict__ post,
                                                    R scale) {
  extern __shared__ unsigned char smem_raw[];
  cplx<R> *sty = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *stz = sty + NY;
  cplx<R> *spost = stz + H;
  cplx<R> *A = spost + (H + 1);
  cplx<R> *B = A + plane_tile(NY, H);
  const int i = blockIdx.x;
  R *data = fb.p[blockIdx.y];
  const cplx<R> *cplane = reinterpret_cast<const cplx<R> *>(data) + (long)i * NY * g.hnz;
  const int nthr = blockDim.x * blockDim.y, lin = threadIdx.y * blockDim.x + threadIdx.x;
  load_table(sty, twy, NY);
  load_table(stz, twz, H);
  load_table(spost, post, H + 1);
  constexpr int ysw = H + 2;
  for (int q = lin; q < NY * (H + 1); q += nthr) {
    const int j = q / (H + 1), k = q - j * (H + 1);
    A[j * ysw + k] = cplane[q];
  }
  __syncthreads();
  const cplx<R> *zres = plane_inv_core<R, NY, H>(A, B, sty, stz, spost);
  constexpr int rsw = NY + 1;
  R *plane = data + (long)i * NY * g.nzp;
  for (int q = lin; q < NY * (H + 1); q += nthr) {
    const int j = q / (H + 1), m = q - j * (H + 1);
    R *rp = plane + (long)j * g.nzp;
    if (m < H) {
      const cplx<R> v = zres[m * rsw + j];
      rp[2 * m] = v.x * scale;
      rp[2 * m + 1] = v.y * scale;
    } else {
      rp[2 * H] = R(0);  // padding of a real-space row
      rp[2 * H + 1] = R(0);
    }
  }
}

// ---- separate passes (planes too large for shared memory) ---------------
// x (axis 0) or y (axis 1) complex pencils, W adjacent pencils per block.
template <typename R, int N, bool INV, int W>
__global__ void __launch_bounds__(512) k_pencils(FieldBatch<R> fb, Grid g, int axis, int tiles_per_row,
                                                 const cplx<R> *__restrict__ tw) {
  extern __shared__ unsigned char smem_raw[];
  const int sw = W + 1;
  cplx<R> *tws = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *ta = tws + N;
  cplx<R> *tb = ta + N * sw;
  cplx<R> *data = reinterpret_cast<cplx<R> *>(fb.p[blockIdx.y]);
  GPencils<R> gp;
  gp.data = data;
  if (axis == 1) {
    const int i = blockIdx.x / tiles_per_row;
    const int kz0 = (blockIdx.x % tiles_per_row) * W;
    gp.base = (long)i * g.ny * g.hnz + kz0;
    gp.pstride = 1;
    gp.estride = g.hnz;
    gp.nvalid = g.hnz - kz0 < W ? g.hnz - kz0 : W;
  } else {
    const long q0 = (long)blockIdx.x * W;
    const long nq = (long)g.ny * g.hnz;
    gp.base = q0;
    gp.pstride = 1;
    gp.estride = nq;
    gp.nvalid = (int)(nq - q0 < W ? nq - q0 : W);
  }
  load_table(tws, tw, N);
  __syncthreads();
  if (INV && axis == 0) {
    GPencilsXInv<R> in{gp, g.ny, g.hnz, g.nx};
    block_fft<R, N, W>(in, gp, ta, tb, sw, tws, true);
  } else {
    block_fft<R, N, W>(gp, gp, ta, tb, sw, tws, INV);
  }
}

// j-direction half of the Hermitian completion (used with the separate
// y pass, before it): per x-plane, columns kz = 0 and kz = NZ/2.
template <typename R>
__global__ void k_herm_columns(FieldBatch<R> fb, Grid g) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int half = g.ny / 2;
  if (t >= (long)g.nx * (half - 1)) return;
  const int i = (int)(t / (half - 1)), j = 1 + (int)(t - (long)i * (half - 1));
  cplx<R> *c = reinterpret_cast<cplx<R> *>(fb.p[blockIdx.y]) + (long)i * g.ny * g.hnz;
  c[(long)(g.ny - j) * g.hnz] = cconj(c[(long)j * g.hnz]);
  c[(long)j * g.hnz + g.hnz - 1] = cconj(c[(long)(g.ny - j) * g.hnz + g.hnz - 1]);
}

// z rows (H = NZ/2), W rows per block.
template <typename R, int H, bool INV, int W>
__global__ void __launch_bounds__(512) k_rows(FieldBatch<R> fb, Grid g, const cplx<R> *__restrict__ tw,
                                              const cplx<R> *__restrict__ post, R scale) {
  extern __shared__ unsigned char smem_raw[];
  const int sw = W + 1;
  cplx<R> *tws = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *spost = tws + H;
  cplx<R> *A = spost + (H + 1);
  cplx<R> *B = A + (H + 2) * sw;
  R *data = fb.p[blockIdx.y];
  const long nrows = (long)g.nx * g.ny;
  const long row0 = (long)blockIdx.x * W;
  const int nthr = blockDim.x * blockDim.y, lin = threadIdx.y * blockDim.x + threadIdx.x;
  load_table(tws, tw, H);
  load_table(spost, post, H + 1);
  constexpr int st = Plan<H>::nstages;
  if (!INV) {
    for (int q = lin; q < W * H; q += nthr) {
      const int w = q / H, e = q - w * H;
      const long row = row0 + w;
      cplx<R> v{0, 0};
      if (row < nrows) {
        const R *rp = data + row * g.nzp;
        v = cplx<R>{rp[2 * e], rp[2 * e + 1]};
      }
      A[e * sw + w] = v;
    }
    __syncthreads();
    cplx<R> *Z = (st & 1) ? B : A;
    block_fft<R, H, W>(SmemT<R>{A, sw}, SmemT<R>{Z, sw}, A, B, sw, tws, false);
    for (int q = lin; q < W * (H + 1); q += nthr) {
      const int w = q / (H + 1), k = q - w * (H + 1);
      const long row = row0 + w;
      if (row >= nrows) continue;
      const int k1 = (k == H) ? 0 : k, k2 = (k == 0) ? 0 : H - k;
      const cplx<R> x = split_fwd(Z[k1 * sw + w], cconj(Z[k2 * sw + w]), spost[k]);
      R *rp = data + row * g.nzp;
      rp[2 * k] = x.x;
      rp[2 * k + 1] = x.y;
    }
  } else {
    for (int q = lin; q < W * (H + 1); q += nthr) {
      const int w = q / (H + 1), k = q - w * (H + 1);
      const long row = row0 + w;
      cplx<R> v{0, 0};
      if (row < nrows) {
        const R *rp = data + row * g.nzp;
        v = cplx<R>{rp[2 * k], (k == 0 || k == H) ? R(0) : rp[2 * k + 1]};
      }
      B[k * sw + w] = v;
    }
    __syncthreads();
    for (int q = lin; q < W * H; q += nthr) {
      const int w = q / H, k = q - w * H;
      A[k * sw + w] = merge_inv(B[k * sw + w], cconj(B[(H - k) * sw + w]), spost[k]);
    }
    __syncthreads();
    cplx<R> *Z = (st & 1) ? B : A;
    block_fft<R, H, W>(SmemT<R>{A, sw}, SmemT<R>{Z, sw}, A, B, sw, tws, true);
    for (int q = lin; q < W * (H + 1); q += nthr) {
      const int w = q / (H + 1), m = q - w * (H + 1);
      const long row = row0 + w;
      if (row >= nrows) continue;
      R *rp = data + row * g.nzp;
      if (m < H) {
        const cplx<R> v = Z[m * sw + w];
        rp[2 * m] = v.x * scale;
        rp[2 * m + 1] = v.y * scale;
      } else {
        rp[2 * H] = R(0);
        rp[2 * H + 1] = R(0);
      }
    }
  }
}

// The residual's z rows in one pass for the three gradient components of the
// float-float operator (blockIdx.y = d): the inverse row transform as k_rows,
// scaled, times the face permittivity 0.5 (eps + eps at the next point along
// d) (the product of refine.cu's eps-face pass, same arithmetic), and the
// forward row transform as k_rows: the real rows stay in shared memory.
template <typename R, int H, int W>
__global__ void __launch_bounds__(512) k_rows_eps(FieldBatch<R> fb, Grid g, const cplx<R> *__restrict__ tw,
                                                  const cplx<R> *__restrict__ post, R scale,
                                                  const float *__restrict__ eps) {
  extern __shared__ unsigned char smem_raw[];
  const int sw = W + 1;
  cplx<R> *tws = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *spost = tws + H;
  cplx<R> *A = spost + (H + 1);
  cplx<R> *B = A + (H + 2) * sw;
  const int d = blockIdx.y;
  R *data = fb.p[0];
#pragma unroll
  for (int c = 1; c < 3; c++)
    if (d == c) data = fb.p[c];
  const long nrows = (long)g.nx * g.ny;
  const long row0 = (long)blockIdx.x * W;
  const int nthr = blockDim.x * blockDim.y, lin = threadIdx.y * blockDim.x + threadIdx.x;
  load_table(tws, tw, H);
  load_table(spost, post, H + 1);
  constexpr int st = Plan<H>::nstages;
  // inverse, as k_rows
  for (int q = lin; q < W * (H + 1); q += nthr) {
    const int w = q / (H + 1), k = q - w * (H + 1);
    const long row = row0 + w;
    cplx<R> v{0, 0};
    if (row < nrows) {
      const R *rp = data + row * g.nzp;
      v = cplx<R>{rp[2 * k], (k == 0 || k == H) ? R(0) : rp[2 * k + 1]};
    }
    B[k * sw + w] = v;
  }
  __syncthreads();
  for (int q = lin; q < W * H; q += nthr) {
    const int w = q / H, k = q - w * H;
    A[k * sw + w] = merge_inv(B[k * sw + w], cconj(B[(H - k) * sw + w]), spost[k]);
  }
  __syncthreads();
  cplx<R> *X = (st & 1) ? B : A;
  block_fft<R, H, W>(SmemT<R>{A, sw}, SmemT<R>{X, sw}, A, B, sw, tws, true);
  // the real row values (2m, 2m+1) at X[m], scaled and times the face
  // permittivity of component d
  // (i, j) of a row by shift and mask (the mesh edges are powers of two),
  // the point and its neighbour along d as row bases plus k
  const int lny = __ffs(g.ny) - 1;
  for (int q = lin; q < W * H; q += nthr) {
    const int w = q / H, m = q - w * H;
    const long row = row0 + w;
    if (row >= nrows) continue;
    const int i = (int)(row >> lny), j = (int)row & (g.ny - 1);
    const long base = row * g.nzp;
    const long nbase = (d == 0)   ? ((long)(((i + 1) & (g.nx - 1)) << lny) + j) * g.nzp
                       : (d == 1) ? ((long)(i << lny) + ((j + 1) & (g.ny - 1))) * g.nzp
                                  : base;
    const cplx<R> v = X[m * sw + w];
    R x[2] = {v.x * scale, v.y * scale};
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int k = 2 * m + h;
      const long im = base + k;
      const long nb = nbase + ((d == 2) ? ((k + 1) & (g.nz - 1)) : k);
      x[h] = x[h] * half_of(two_sum(eps[im], eps[nb]));
    }
    X[m * sw + w] = cplx<R>{x[0], x[1]};
  }
  __syncthreads();
  // forward, as k_rows, from X (the other tile the ping-pong partner)
  cplx<R> *Y = (X == A) ? B : A;
  cplx<R> *Z = (st & 1) ? Y : X;
  block_fft<R, H, W>(SmemT<R>{X, sw}, SmemT<R>{Z, sw}, X, Y, sw, tws, false);
  for (int q = lin; q < W * (H + 1); q += nthr) {
    const int w = q / (H + 1), k = q - w * (H + 1);
    const long row = row0 + w;
    if (row >= nrows) continue;
    const int k1 = (k == H) ? 0 : k, k2 = (k == 0) ? 0 : H - k;
    const cplx<R> xo = split_fwd(Z[k1 * sw + w], cconj(Z[k2 * sw + w]), spost[k]);
    R *rp = data + row * g.nzp;
    rp[2 * k] = xo.x;
    rp[2 * k + 1] = xo.y;
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
R table_value(long double v) {
  return (R)v;
}
template <>
dfl table_value<dfl>(long double v) {
  const float h = (float)v;
  return dfl(h, (float)(v - (long double)h));
}

template <typename R>
cplx<R> *upload_table(int n, int denom, cudaStream_t s) {
  std::vector<cplx<R>> h(n);
  for (int m = 0; m < n; m++) {
    long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)m / (long double)denom;
    h[m].x = table_value<R>(cosl(a));
    h[m].y = table_value<R>(sinl(a));
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

// ---- launch helpers -------------------------------------------------------
constexpr size_t PLANE_SMEM_MAX = 200 * 1024;

template <typename R>
size_t plane_smem(int ny, int h) {
  return ((size_t)ny + h + (h + 1) + 2 * (size_t)plane_tile(ny, h)) * sizeof(cplx<R>);
}
template <typename R>
size_t pencil_smem(int n) {
  return ((size_t)n + 2 * (size_t)n * (pencil_width<R>() + 1)) * sizeof(cplx<R>);
}
template <typename R>
constexpr int row_width() {
  return 2 * pencil_width<R>();
}
template <typename R>
size_t row_smem(int h) {
  return ((size_t)h + (h + 1) + 2 * (size_t)(h + 2) * (row_width<R>() + 1)) * sizeof(cplx<R>);
}

// The float-float transforms run the separate passes only: at 128^3 an
// x-plane of an 8-byte type exceeds shared memory anyway, and the plane
// kernels' compile time in float-float arithmetic is prohibitive.
template <typename R>
constexpr bool has_plane_kernels() {
  return !std::is_same<R, dfl>::value;
}

template <typename R>
bool use_plane(const Grid &g) {
  return g.ny <= 128 && g.nz <= 128 && plane_smem<R>(g.ny, g.nz / 2) <= PLANE_SMEM_MAX;
}

template <typename R, int NY, int H>
void launch_plane_nh(const FFTPlan<R> &p, const FieldBatch<R> &fb, bool inverse, cudaStream_t s) {
  if constexpr (std::is_same<R, float>::value) {
    if (fft_plane_r(p, fb, inverse, s)) return;  // the register-resident kernels (kop.cu)
  }
  const size_t sm = plane_smem<R>(NY, H);
  count_launch(fld<R>(p.g, 1.0 * fb.n));
  if (!inverse) {
    k_plane_fwd<R, NY, H><<<dim3(p.g.nx, fb.n), 1024, sm, s>>>(fb, p.g, p.tw_y, p.tw_z, p.tw_post);
  } else {
    const R scale = from_double<R>(1.0 / ((double)p.g.nx * p.g.ny * p.g.nz));
    k_plane_inv<R, NY, H><<<dim3(p.g.nx, fb.n), 1024, sm, s>>>(fb, p.g, p.tw_y, p.tw_z, p.tw_post, scale);
  }
}

template <typename R, int NY>
void launch_plane_n(const FFTPlan<R> &p, const FieldBatch<R> &fb, bool inverse, cudaStream_t s) {
  switch (p.g.nz / 2) {
    case 8: launch_plane_nh<R, NY, 8>(p, fb, inverse, s); break;
    case 16: launch_plane_nh<R, NY, 16>(p, fb, inverse, s); break;
    case 32: launch_plane_nh<R, NY, 32>(p, fb, inverse, s); break;
    default: launch_plane_nh<R, NY, 64>(p, fb, inverse, s); break;
  }
}

template <typename R>
void launch_plane(const FFTPlan<R> &p, const FieldBatch<R> &fb, bool inverse, cudaStream_t s) {
  switch (p.g.ny) {
    case 16: launch_plane_n<R, 16>(p, fb, inverse, s); break;
    case 32: launch_plane_n<R, 32>(p, fb, inverse, s); break;
    case 64: launch_plane_n<R, 64>(p, fb, inverse, s); break;
    default: launch_plane_n<R, 128>(p, fb, inverse, s); break;
  }
}

template <typename R, int N>
void launch_pencils_n(const FFTPlan<R> &p, const FieldBatch<R> &fb, int axis, bool inverse, cudaStream_t s) {
  const Grid &g = p.g;
  constexpr int W = pencil_width<R>();
  const int tiles_per_row = (g.hnz + W - 1) / W;
  const unsigned nblk = axis == 1 ? (unsigned)(g.nx * tiles_per_row) : div_up((long)g.ny * g.hnz, W);
  const dim3 block(W, N / 8 < 512 / W ? N / 8 : 512 / W);
  count_launch(fld<R>(g, (axis == 0 ? 1.0 : 0.5) * fb.n));
  const cplx<R> *tw = axis == 0 ? p.tw_x : p.tw_y;
  if (inverse)
    k_pencils<R, N, true, W><<<dim3(nblk, fb.n), block, pencil_smem<R>(N), s>>>(fb, g, axis, tiles_per_row, tw);
  else
    k_pencils<R, N, false, W><<<dim3(nblk, fb.n), block, pencil_smem<R>(N), s>>>(fb, g, axis, tiles_per_row, tw);
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
  const dim3 block(W, H / 8 < 512 / W ? H / 8 : 512 / W);
  const R scale = from_double<R>(1.0 / ((double)g.nx * g.ny * g.nz));
  count_launch(fld<R>(g, 0.5 * fb.n));
  if (inverse) k_rows<R, H, true, W><<<grid, block, row_smem<R>(H), s>>>(fb, g, p.tw_z, p.tw_post, scale);
  else k_rows<R, H, false, W><<<grid, block, row_smem<R>(H), s>>>(fb, g, p.tw_z, p.tw_post, scale);
}

template <typename R, int H>
void launch_rows_eps_n(const FFTPlan<R> &p, const FieldBatch<R> &fb, const float *eps, cudaStream_t s) {
  const Grid &g = p.g;
  constexpr int W = row_width<R>();
  static bool attr = false;  // one attribute call per instantiation
  if (!attr) {
    cudaFuncSetAttribute(k_rows_eps<R, H, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)row_smem<R>(H));
    attr = true;
  }
  const dim3 grid(div_up((long)g.nx * g.ny, W), 3);
  const dim3 block(W, H / 8 < 512 / W ? H / 8 : 512 / W);
  const R scale = from_double<R>(1.0 / ((double)g.nx * g.ny * g.nz));
  // the two half passes of each field and the permittivity read
  count_launch(fld<R>(g, 3.0) + fld<float>(g, 1.0));
  k_rows_eps<R, H, W><<<grid, block, row_smem<R>(H), s>>>(fb, g, p.tw_z, p.tw_post, scale, eps);
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
void launch_herm_columns(const FFTPlan<R> &p, const FieldBatch<R> &fb, cudaStream_t s) {
  const long n = (long)p.g.nx * (p.g.ny / 2 - 1);
  count_launch();
  k_herm_columns<R><<<dim3(div_up(n, 256), fb.n), 256, 0, s>>>(fb, p.g);
}

template <typename R, int NY, int H>
void set_plane_attr() {
  cudaFuncSetAttribute(k_plane_fwd<R, NY, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plane_smem<R>(NY, H));
  cudaFuncSetAttribute(k_plane_inv<R, NY, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plane_smem<R>(NY, H));
}
template <typename R, int N>
void set_pencil_attr() {
  constexpr int W = pencil_width<R>();
  cudaFuncSetAttribute(k_pencils<R, N, false, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pencil_smem<R>(N));
  cudaFuncSetAttribute(k_pencils<R, N, true, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pencil_smem<R>(N));
}
template <typename R, int H>
void set_row_attr() {
  constexpr int W = row_width<R>();
  cudaFuncSetAttribute(k_rows<R, H, false, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)row_smem<R>(H));
  cudaFuncSetAttribute(k_rows<R, H, true, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)row_smem<R>(H));
}

template <typename R, int NY>
void set_plane_attr_ny(int h) {
  switch (h) {
    case 8: set_plane_attr<R, NY, 8>(); break;
    case 16: set_plane_attr<R, NY, 16>(); break;
    case 32: set_plane_attr<R, NY, 32>(); break;
    default: set_plane_attr<R, NY, 64>(); break;
  }
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
  if constexpr (has_plane_kernels<R>()) {
    if (use_plane<R>(g)) {
      switch (g.ny) {
        case 16: set_plane_attr_ny<R, 16>(g.nz / 2); break;
        case 32: set_plane_attr_ny<R, 32>(g.nz / 2); break;
        case 64: set_plane_attr_ny<R, 64>(g.nz / 2); break;
        default: set_plane_attr_ny<R, 128>(g.nz / 2); break;
      }
    }
  }
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
  fft_pass(p, fb, 0, s);
  fft_pass(p, fb, 1, s);
}

template <typename R>
void fft_c2r(const FFTPlan<R> &p, const FieldBatch<R> &fb, cudaStream_t s) {
  fft_pass(p, fb, 2, s);
  fft_pass(p, fb, 3, s);
}

template <typename R>
void fft_c2r_eps_r2c(const FFTPlan<R> &p, const FieldBatch<R> &fb, const float *eps, cudaStream_t s) {
  launch_pencils(p, fb, 0, true, s);  // x inverse
  launch_herm_columns(p, fb, s);
  launch_pencils(p, fb, 1, true, s);  // y inverse
  switch (p.g.nz / 2) {               // z rows inverse, the product, z rows forward
    case 8: launch_rows_eps_n<R, 8>(p, fb, eps, s); break;
    case 16: launch_rows_eps_n<R, 16>(p, fb, eps, s); break;
    case 32: launch_rows_eps_n<R, 32>(p, fb, eps, s); break;
    case 64: launch_rows_eps_n<R, 64>(p, fb, eps, s); break;
    default: launch_rows_eps_n<R, 128>(p, fb, eps, s); break;
  }
  launch_pencils(p, fb, 1, false, s);  // y forward
  launch_pencils(p, fb, 0, false, s);  // x forward
}

template <typename R>
void fft_pass(const FFTPlan<R> &p, const FieldBatch<R> &fb, int pass, cudaStream_t s) {
  if constexpr (has_plane_kernels<R>()) {
    if (use_plane<R>(p.g) && (pass == 0 || pass == 3)) {
      launch_plane(p, fb, pass == 3, s);  // 0: z rows + y pencils forward; 3: y pencils + z rows inverse
      return;
    }
  }
  switch (pass) {
    case 0:  // z rows + y pencils, forward
      launch_rows(p, fb, false, s);
      launch_pencils(p, fb, 1, false, s);
      break;
    case 1: launch_pencils(p, fb, 0, false, s); break;  // x pencils, forward
    case 2: launch_pencils(p, fb, 0, true, s); break;   // x pencils, inverse
    default:                                            // y pencils + z rows, inverse
      launch_herm_columns(p, fb, s);
      launch_pencils(p, fb, 1, true, s);
      launch_rows(p, fb, true, s);
  }
}

}  // namespace icep
