// fft.cu -- batched 3D real FFT kernels (see fft.cuh).
#include <math.h>
#include <vector>

#include "fft.cuh"

namespace icep {

namespace {

template <typename R>
__device__ __forceinline__ cplx<R> cmul(cplx<R> a, cplx<R> b) {
  cplx<R> r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

// Stockham radix-2 sweep over W pencils of length n held element-major in
// shared memory (element e of pencil w at s[e*W + w]). Each of the T threads of
// pencil w handles butterflies tid, tid+T, ... < n/2. Forward kernel
// exp(-2 pi i / n) from tw (n entries); inverse uses the conjugate. Returns the
// buffer that holds the result (a or b). Every thread of the block calls it.
template <typename R>
__device__ cplx<R> *stockham(cplx<R> *a, cplx<R> *b, int n, int W, int w, int tid, int T,
                             const cplx<R> *__restrict__ tw, bool inverse) {
  cplx<R> *src = a, *dst = b;
  const int half = n >> 1;
  for (int ls = 1; ls < n; ls <<= 1) {
    const int twstep = n / (2 * ls);
    for (int j = tid; j < half; j += T) {
      const int p = j & (ls - 1);
      const int k = j - p;  // (j / ls) * ls
      cplx<R> x0 = src[j * W + w];
      cplx<R> x1 = src[(j + half) * W + w];
      cplx<R> wv = tw[p * twstep];
      if (inverse) wv.y = -wv.y;
      cplx<R> t = cmul(wv, x1);
      const int o = 2 * k + p;
      dst[o * W + w] = cplx<R>{x0.x + t.x, x0.y + t.y};
      dst[(o + ls) * W + w] = cplx<R>{x0.x - t.x, x0.y - t.y};
    }
    __syncthreads();
    cplx<R> *tmp = src;
    src = dst;
    dst = tmp;
  }
  return src;
}

// Complex FFT along y (axis 1) or x (axis 0) for W pencils per block.
template <typename R>
__global__ void k_pencils(FieldBatch<R> fb, Grid g, int axis, int W, int tiles_per_row,
                          const cplx<R> *__restrict__ tw, int inverse) {
  extern __shared__ unsigned char smem_raw[];
  const int n = (axis == 0) ? g.nx : g.ny;
  cplx<R> *sa = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *sb = sa + n * W;
  cplx<R> *data = reinterpret_cast<cplx<R> *>(fb.p[blockIdx.y]);
  const int w = threadIdx.x, tid = threadIdx.y, T = blockDim.y;
  long base;
  long stride;
  bool valid;
  if (axis == 1) {
    // pencil (i, kz): start i*NY*hnz + kz, stride hnz
    const int i = blockIdx.x / tiles_per_row;
    const int kz = (blockIdx.x % tiles_per_row) * W + w;
    valid = kz < g.hnz;
    base = (long)i * g.ny * g.hnz + kz;
    stride = g.hnz;
  } else {
    // pencil q = j*hnz + kz: start q, stride NY*hnz
    const long q = (long)blockIdx.x * W + w;
    valid = q < (long)g.ny * g.hnz;
    base = q;
    stride = (long)g.ny * g.hnz;
  }
  for (int e = tid; e < n; e += T) sa[e * W + w] = valid ? data[base + e * stride] : cplx<R>{0, 0};
  __syncthreads();
  cplx<R> *res = stockham(sa, sb, n, W, w, tid, T, tw, inverse != 0);
  if (valid)
    for (int e = tid; e < n; e += T) data[base + e * stride] = res[e * W + w];
}

// z rows, forward: NZ reals -> NZ/2+1 complex via an NZ/2-point complex FFT
// of z[m] = x[2m] + i x[2m+1] and the split X[k] = E[k] + exp(-2 pi i k/NZ) O[k].
template <typename R>
__global__ void k_rows_r2c(FieldBatch<R> fb, Grid g, int W, const cplx<R> *__restrict__ tw,
                           const cplx<R> *__restrict__ post) {
  extern __shared__ unsigned char smem_raw[];
  const int h = g.nz / 2;
  cplx<R> *sa = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *sb = sa + h * W;
  R *data = fb.p[blockIdx.y];
  const long nrows = (long)g.nx * g.ny;
  const long row0 = (long)blockIdx.x * W;
  const int nthr = blockDim.x * blockDim.y;
  const int lin = threadIdx.y * blockDim.x + threadIdx.x;
  // coalesced load of W rows (h complex each)
  for (int q = lin; q < W * h; q += nthr) {
    const int w = q / h, e = q - (q / h) * h;
    const long row = row0 + w;
    cplx<R> v{0, 0};
    if (row < nrows) {
      const R *rp = data + row * g.nzp;
      v.x = rp[2 * e];
      v.y = rp[2 * e + 1];
    }
    sa[e * W + w] = v;
  }
  __syncthreads();
  const int w = threadIdx.x, tid = threadIdx.y, T = blockDim.y;
  cplx<R> *Z = stockham(sa, sb, h, W, w, tid, T, tw, false);
  // split into the half spectrum; written back in place (this block's rows only)
  for (int q = lin; q < W * (h + 1); q += nthr) {
    const int wr = q / (h + 1), k = q - wr * (h + 1);
    const long row = row0 + wr;
    if (row >= nrows) continue;
    const int k1 = (k == h) ? 0 : k, k2 = (k == 0) ? 0 : h - k;
    cplx<R> z = Z[k1 * W + wr];
    cplx<R> c = Z[k2 * W + wr];
    c.y = -c.y;
    const R er = R(0.5) * (z.x + c.x), ei = R(0.5) * (z.y + c.y);
    const R orr = R(0.5) * (z.y - c.y), oi = R(-0.5) * (z.x - c.x);
    const cplx<R> pw = post[k];
    R *rp = data + row * g.nzp;
    rp[2 * k] = er + (pw.x * orr - pw.y * oi);
    rp[2 * k + 1] = ei + (pw.x * oi + pw.y * orr);
  }
}

// z rows, inverse: half spectrum -> NZ reals, scaled. Imaginary parts of
// kz = 0 and kz = NZ/2 are ignored (as in a standard real inverse).
template <typename R>
__global__ void k_rows_c2r(FieldBatch<R> fb, Grid g, int W, const cplx<R> *__restrict__ tw,
                           const cplx<R> *__restrict__ post, R scale) {
  extern __shared__ unsigned char smem_raw[];
  const int h = g.nz / 2;
  cplx<R> *sa = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *sb = sa + h * W;
  cplx<R> *sx = sb + h * W;  // staged half spectrum, (h+1) per row
  R *data = fb.p[blockIdx.y];
  const long nrows = (long)g.nx * g.ny;
  const long row0 = (long)blockIdx.x * W;
  const int nthr = blockDim.x * blockDim.y;
  const int lin = threadIdx.y * blockDim.x + threadIdx.x;
  for (int q = lin; q < W * (h + 1); q += nthr) {
    const int w = q / (h + 1), k = q - w * (h + 1);
    const long row = row0 + w;
    cplx<R> v{0, 0};
    if (row < nrows) {
      const R *rp = data + row * g.nzp;
      v.x = rp[2 * k];
      v.y = (k == 0 || k == h) ? R(0) : rp[2 * k + 1];
    }
    sx[w * (h + 1) + k] = v;
  }
  __syncthreads();
  for (int q = lin; q < W * h; q += nthr) {
    const int w = q / h, k = q - w * h;
    const cplx<R> x = sx[w * (h + 1) + k];
    cplx<R> c = sx[w * (h + 1) + (h - k)];
    c.y = -c.y;
    const R sr = x.x + c.x, si = x.y + c.y;
    const R dr = x.x - c.x, di = x.y - c.y;
    const cplx<R> pw = post[k];  // exp(-2 pi i k/NZ); use its conjugate
    const R wr = pw.x, wi = -pw.y;
    const R tr = wr * dr - wi * di, ti = wr * di + wi * dr;
    sa[k * W + w] = cplx<R>{sr - ti, si + tr};
  }
  __syncthreads();
  const int w = threadIdx.x, tid = threadIdx.y, T = blockDim.y;
  cplx<R> *z = stockham(sa, sb, h, W, w, tid, T, tw, true);
  for (int q = lin; q < W * h; q += nthr) {
    const int wr = q / h, m = q - wr * h;
    const long row = row0 + wr;
    if (row >= nrows) continue;
    R *rp = data + row * g.nzp;
    const cplx<R> v = z[m * W + wr];
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
int pencil_width() {
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

}  // namespace

template <typename R>
int fft_plan_init(FFTPlan<R> &p, const Grid &g, cudaStream_t s) {
  p.g = g;
  p.tw_x = upload_table<R>(g.nx, g.nx, s);
  p.tw_y = upload_table<R>(g.ny, g.ny, s);
  p.tw_z = upload_table<R>(g.nz / 2, g.nz / 2, s);
  p.tw_post = upload_table<R>(g.nz / 2 + 1, g.nz, s);
  if (!p.tw_x || !p.tw_y || !p.tw_z || !p.tw_post) return ICEP_ERR_CUDA;
  const int W = pencil_width<R>();
  const int WR = 2 * W;  // rows per block of the z-row kernels
  const size_t sm_pen = 2 * (size_t)((g.nx > g.ny) ? g.nx : g.ny) * W * sizeof(cplx<R>);
  const size_t sm_row = (2 * (size_t)(g.nz / 2) * WR + (size_t)WR * (g.nz / 2 + 1)) * sizeof(cplx<R>);
  cudaFuncSetAttribute(k_pencils<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_pen);
  cudaFuncSetAttribute(k_rows_r2c<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_row);
  cudaFuncSetAttribute(k_rows_c2r<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_row);
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

namespace {
template <typename R>
void launch_pencils(const FFTPlan<R> &p, const FieldBatch<R> &fb, int axis, bool inverse, cudaStream_t s) {
  const Grid &g = p.g;
  const int W = pencil_width<R>();
  const int n = axis == 0 ? g.nx : g.ny;
  int T = n / 2;
  if (T * W > 1024) T = 1024 / W;
  dim3 block(W, T);
  int tiles_per_row = (g.hnz + W - 1) / W;
  unsigned nblk = axis == 1 ? (unsigned)(g.nx * tiles_per_row) : div_up((long)g.ny * g.hnz, W);
  dim3 grid(nblk, fb.n);
  size_t sm = 2 * (size_t)n * W * sizeof(cplx<R>);
  k_pencils<R><<<grid, block, sm, s>>>(fb, g, axis, W, tiles_per_row, axis == 0 ? p.tw_x : p.tw_y,
                                        inverse ? 1 : 0);
}

template <typename R>
void row_launch_dims(const Grid &g, int &W, dim3 &block, dim3 &grid, int nb) {
  W = pencil_width<R>() * 2;
  const int h = g.nz / 2;
  int T = h / 2 > 0 ? h / 2 : 1;
  if (T * W > 1024) T = 1024 / W;
  block = dim3(W, T);
  grid = dim3(div_up((long)g.nx * g.ny, W), nb);
}
}  // namespace

template <typename R>
void fft_r2c(const FFTPlan<R> &p, const FieldBatch<R> &fb, cudaStream_t s) {
  const Grid &g = p.g;
  int W;
  dim3 block, grid;
  row_launch_dims<R>(g, W, block, grid, fb.n);
  size_t sm = (2 * (size_t)(g.nz / 2) * W + (size_t)W * (g.nz / 2 + 1)) * sizeof(cplx<R>);
  k_rows_r2c<R><<<grid, block, sm, s>>>(fb, g, W, p.tw_z, p.tw_post);
  launch_pencils(p, fb, 1, false, s);
  launch_pencils(p, fb, 0, false, s);
}

template <typename R>
void fft_c2r(const FFTPlan<R> &p, const FieldBatch<R> &fb, cudaStream_t s) {
  const Grid &g = p.g;
  {
    long n = 2L * g.nx * g.ny;
    k_herm_project<R><<<dim3(div_up(n, 256), fb.n), 256, 0, s>>>(fb, g);
  }
  launch_pencils(p, fb, 0, true, s);
  launch_pencils(p, fb, 1, true, s);
  int W;
  dim3 block, grid;
  row_launch_dims<R>(g, W, block, grid, fb.n);
  size_t sm = (2 * (size_t)(g.nz / 2) * W + (size_t)W * (g.nz / 2 + 1)) * sizeof(cplx<R>);
  const R scale = (R)(1.0 / ((double)g.nx * g.ny * g.nz));
  k_rows_c2r<R><<<grid, block, sm, s>>>(fb, g, W, p.tw_z, p.tw_post, scale);
}

template int fft_plan_init<double>(FFTPlan<double> &, const Grid &, cudaStream_t);
template int fft_plan_init<float>(FFTPlan<float> &, const Grid &, cudaStream_t);
template void fft_plan_free<double>(FFTPlan<double> &);
template void fft_plan_free<float>(FFTPlan<float> &);
template void fft_r2c<double>(const FFTPlan<double> &, const FieldBatch<double> &, cudaStream_t);
template void fft_r2c<float>(const FFTPlan<float> &, const FieldBatch<float> &, cudaStream_t);
template void fft_c2r<double>(const FFTPlan<double> &, const FieldBatch<double> &, cudaStream_t);
template void fft_c2r<float>(const FFTPlan<float> &, const FieldBatch<float> &, cudaStream_t);

}  // namespace icep
