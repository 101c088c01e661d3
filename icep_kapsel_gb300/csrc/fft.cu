// fft.cu -- batched 3D real FFT kernels (see fft.cuh).
//
// Every 1D transform is a Stockham autosort FFT with radix-8/4/2 stages held
// in registers (block_fft): a pencil of N complex values is split into N/8
// work items per stage, each one radix-8 (or two radix-4, four radix-2)
// butterflies; the items of all pencils a block owns are spread over its
// threads, and stages exchange data through padded shared-memory tiles
// (element e of pencil w at tile[e*sw + w], conflict-free). The inverse is
// conj(FFT(conj(x))), so only forward butterflies and twiddles exist.
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
__device__ __forceinline__ cplx<R> cconj(cplx<R> a) { return cplx<R>{a.x, -a.y}; }
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

// ---- stage sources and sinks --------------------------------------------
template <typename R>
struct SmemT {  // shared tile, element e of pencil w at t[e*sw + w]
  cplx<R> *t;
  int sw;
  __device__ __forceinline__ cplx<R> load(int w, int e) const { return t[e * sw + w]; }
  __device__ __forceinline__ void store(int w, int e, cplx<R> v) const { t[e * sw + w] = v; }
};

template <typename R>
struct GPencils {  // global pencils: element e of pencil w at data[base + w*pstride + e*estride]
  cplx<R> *data;
  long base, pstride, estride;
  int nvalid;
  __device__ __forceinline__ cplx<R> load(int w, int e) const {
    return (w < nvalid) ? data[base + w * pstride + e * estride] : cplx<R>{0, 0};
  }
  __device__ __forceinline__ void store(int w, int e, cplx<R> v) const {
    if (w < nvalid) data[base + w * pstride + e * estride] = v;
  }
};

// x pencils of the inverse transform. The pencils (j, kz) with j in {0, NY/2}
// and kz in {0, NZ/2} get the i-direction half of the reference's Hermitian
// completion as they are read: kz = 0 keeps i <= NX/2, kz = NZ/2 keeps
// i > NX/2, the other entries read conj(X(NX - i)); i in {0, NX/2} keep their
// real part. Reads come straight from global memory, and the pass writes
// its output only after the first stage has finished everywhere.
template <typename R>
struct GPencilsXInv {
  GPencils<R> g;
  int ny, hnz, nx;
  __device__ __forceinline__ cplx<R> load(int w, int e) const {
    if (w >= g.nvalid) return cplx<R>{0, 0};
    const long q = g.base + w;  // pencil index j*hnz + kz
    const int j = (int)(q / hnz), kz = (int)(q - (long)j * hnz);
    const cplx<R> v = g.data[q + e * g.estride];
    if ((j == 0 || j == ny / 2) && (kz == 0 || kz == hnz - 1)) {
      if (e == 0 || e == nx / 2) return cplx<R>{v.x, R(0)};
      const bool kept = (kz == 0) ? (e <= nx / 2) : (e > nx / 2);
      if (!kept) return cconj(g.data[q + (nx - e) * g.estride]);
    }
    return v;
  }
  __device__ __forceinline__ void store(int w, int e, cplx<R> v) const { g.store(w, e, v); }
};

// One Stockham stage of radix RAD over Wp pencils. Ls: product of the
// previous radices. Item jb of pencil w reads elements jb + q*N/RAD, applies
// twiddles exp(-2 pi i p q/(Ls RAD)), and writes k*Ls*RAD + p + Ls*q
// (jb = k*Ls + p). Items are distributed over all threads of the block, the
// pencil index fastest (coalesced global access for adjacent pencils).
template <typename R, int N, int RAD, int WP, class Src, class Dst>
__device__ __forceinline__ void stage(const Src &src, const Dst &dst, int Ls, const cplx<R> *__restrict__ tws,
                                      bool conj_in, bool conj_out) {
  constexpr int T = N / 8;
  constexpr int NB = 8 / RAD;
  const int nthr = blockDim.x * blockDim.y;
  const int lin = threadIdx.y * blockDim.x + threadIdx.x;
  constexpr int items = WP * T;
  for (int it = lin; it < items; it += nthr) {
    const int w = it % WP, tid = it / WP;
#pragma unroll
    for (int m = 0; m < NB; m++) {
      const int jb = tid + T * m;
      const int p = jb & (Ls - 1);
      const int k = jb / Ls;
      cplx<R> v[RAD];
#pragma unroll
      for (int q = 0; q < RAD; q++) v[q] = conj_if(src.load(w, jb + q * (N / RAD)), conj_in);
      if (Ls > 1) {
        const int step = N / (Ls * RAD);
#pragma unroll
        for (int q = 1; q < RAD; q++) v[q] = cmul(v[q], tws[(p * q * step) & (N - 1)]);
      }
      dftr<R, RAD>(v);
#pragma unroll
      for (int q = 0; q < RAD; q++) dst.store(w, k * Ls * RAD + p + Ls * q, conj_if(v[q], conj_out));
    }
  }
}

// Length-N transforms of Wp pencils. The first stage reads `in`, the last
// writes `out`; intermediate stages alternate between tiles a and b (both of
// stride sw). A __syncthreads follows every stage.
template <typename R, int N, int WP, class In, class Out>
__device__ __forceinline__ void block_fft(const In &in, const Out &out, cplx<R> *a, cplx<R> *b, int sw,
                                          const cplx<R> *tws, bool inverse) {
  SmemT<R> ta{a, sw}, tb{b, sw};
  int Ls = 1;
#pragma unroll
  for (int s = 0; s < Plan<N>::nstages; s++) {
    const int rad = Plan<N>::radix(s);
    const bool first = (s == 0), last = (s == Plan<N>::nstages - 1);
    const bool ci = first && inverse, co = last && inverse;
    const SmemT<R> &tsrc = (s & 1) ? tb : ta;
    const SmemT<R> &tdst = (s & 1) ? ta : tb;
    if (first && last) {
      if (rad == 8) stage<R, N, 8, WP>(in, out, Ls, tws, ci, co);
    } else if (first) {
      if (rad == 8) stage<R, N, 8, WP>(in, tb, Ls, tws, ci, co);
      else if (rad == 4) stage<R, N, 4, WP>(in, tb, Ls, tws, ci, co);
      else stage<R, N, 2, WP>(in, tb, Ls, tws, ci, co);
    } else if (last) {
      if (rad == 8) stage<R, N, 8, WP>(tsrc, out, Ls, tws, ci, co);
      else if (rad == 4) stage<R, N, 4, WP>(tsrc, out, Ls, tws, ci, co);
      else stage<R, N, 2, WP>(tsrc, out, Ls, tws, ci, co);
    } else {
      if (rad == 8) stage<R, N, 8, WP>(tsrc, tdst, Ls, tws, ci, co);
      else if (rad == 4) stage<R, N, 4, WP>(tsrc, tdst, Ls, tws, ci, co);
      else stage<R, N, 2, WP>(tsrc, tdst, Ls, tws, ci, co);
    }
    Ls *= rad;
    __syncthreads();
  }
}

template <typename R>
__device__ __forceinline__ void load_table(cplx<R> *dst, const cplx<R> *__restrict__ src, int n) {
  const int lin = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  for (int q = lin; q < n; q += nthr) dst[q] = src[q];
}

// z row split/merge of the real transform (H = NZ/2):
//   forward  X[k] = E[k] + exp(-2 pi i k/NZ) O[k],  E, O from Z[k], conj Z[H-k]
//   inverse  Z[k] = (X[k] + conj X[H-k]) + i exp(+2 pi i k/NZ)(X[k] - conj X[H-k])
template <typename R>
__device__ __forceinline__ cplx<R> split_fwd(cplx<R> z, cplx<R> c /* conj Z[H-k] */, cplx<R> pw) {
  const R er = R(0.5) * (z.x + c.x), ei = R(0.5) * (z.y + c.y);
  const R orr = R(0.5) * (z.y - c.y), oi = R(-0.5) * (z.x - c.x);
  return cplx<R>{er + (pw.x * orr - pw.y * oi), ei + (pw.x * oi + pw.y * orr)};
}
template <typename R>
__device__ __forceinline__ cplx<R> merge_inv(cplx<R> x, cplx<R> c /* conj X[H-k] */, cplx<R> pw) {
  const R sr = x.x + c.x, si = x.y + c.y;
  const R dr = x.x - c.x, di = x.y - c.y;
  const R wr = pw.x, wi = -pw.y;  // exp(+2 pi i k/NZ)
  const R tr = wr * dr - wi * di, ti = wr * di + wi * dr;
  return cplx<R>{sr - ti, si + tr};
}

// ---- plane kernels (one block per x-plane and field) ---------------------
// smem: tw_y[NY] | tw_z[H] | post[H+1] | A | B, A/B of plane_tile() complex.
__host__ __device__ constexpr int plane_tile(int ny, int h) {
  return (h * (ny + 1) > ny * (h + 2)) ? h * (ny + 1) : ny * (h + 2);
}

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
  // z transforms: A -> (B, ...); with an even number of stages the result is in A
  constexpr int zst = Plan<H>::nstages;
  cplx<R> *zres = (zst & 1) ? B : A;
  cplx<R> *ybuf = (zst & 1) ? A : B;
  block_fft<R, H, NY>(SmemT<R>{A, rsw}, SmemT<R>{zres, rsw}, A, B, rsw, stz, false);
  // split into the half spectrum, y-pencil layout: element j of pencil k at ybuf[j*ysw + k]
  constexpr int ysw = H + 2;
  for (int q = lin; q < NY * (H + 1); q += nthr) {
    const int j = q / (H + 1), k = q - j * (H + 1);
    const int k1 = (k == H) ? 0 : k, k2 = (k == 0) ? 0 : H - k;
    ybuf[j * ysw + k] = split_fwd(zres[k1 * rsw + j], cconj(zres[k2 * rsw + j]), spost[k]);
  }
  __syncthreads();
  // y transforms of the H+1 columns, last stage to global (coalesced over kz)
  GPencils<R> outp{reinterpret_cast<cplx<R> *>(data), (long)i * NY * g.hnz, 1, g.hnz, H + 1};
  cplx<R> *other = (ybuf == A) ? B : A;
  block_fft<R, NY, H + 1>(SmemT<R>{ybuf, ysw}, outp, ybuf, other, ysw, sty, false);
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
  // j-direction half of the Hermitian completion on the kz = 0 and kz = NZ/2
  // columns: kz = 0 keeps rows 1..NY/2-1, kz = NZ/2 keeps rows NY/2+1..NY-1.
  for (int j = 1 + lin; j < NY / 2; j += nthr) {
    A[(NY - j) * ysw + 0] = cconj(A[j * ysw + 0]);
    A[j * ysw + H] = cconj(A[(NY - j) * ysw + H]);
  }
  __syncthreads();
  // y inverse transforms of the H+1 columns
  constexpr int yst = Plan<NY>::nstages;
  cplx<R> *yres = (yst & 1) ? B : A;
  cplx<R> *zbuf = (yst & 1) ? A : B;
  block_fft<R, NY, H + 1>(SmemT<R>{A, ysw}, SmemT<R>{yres, ysw}, A, B, ysw, sty, true);
  // merge into H-point complex rows (element-major, pencil = row j); the
  // imaginary parts of kz = 0 and kz = NZ/2 are ignored
  constexpr int rsw = NY + 1;
  for (int q = lin; q < NY * H; q += nthr) {
    const int j = q / H, k = q - j * H;
    cplx<R> x = yres[j * ysw + k];
    cplx<R> c = yres[j * ysw + (H - k)];
    if (k == 0) {
      x.y = R(0);
      c.y = R(0);
    }
    zbuf[k * rsw + j] = merge_inv(x, cconj(c), spost[k]);
  }
  __syncthreads();
  constexpr int zst = Plan<H>::nstages;
  cplx<R> *other = (zbuf == A) ? B : A;
  cplx<R> *zres = (zst & 1) ? other : zbuf;
  block_fft<R, H, NY>(SmemT<R>{zbuf, rsw}, SmemT<R>{zres, rsw}, zbuf, other, rsw, stz, true);
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

template <typename R>
bool use_plane(const Grid &g) {
  return g.ny <= 128 && g.nz <= 128 && plane_smem<R>(g.ny, g.nz / 2) <= PLANE_SMEM_MAX;
}

template <typename R, int NY, int H>
void launch_plane_nh(const FFTPlan<R> &p, const FieldBatch<R> &fb, bool inverse, cudaStream_t s) {
  const size_t sm = plane_smem<R>(NY, H);
  count_launch();
  if (!inverse) {
    k_plane_fwd<R, NY, H><<<dim3(p.g.nx, fb.n), 1024, sm, s>>>(fb, p.g, p.tw_y, p.tw_z, p.tw_post);
  } else {
    const R scale = (R)(1.0 / ((double)p.g.nx * p.g.ny * p.g.nz));
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
  count_launch();
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
  const R scale = (R)(1.0 / ((double)g.nx * g.ny * g.nz));
  count_launch();
  if (inverse) k_rows<R, H, true, W><<<grid, block, row_smem<R>(H), s>>>(fb, g, p.tw_z, p.tw_post, scale);
  else k_rows<R, H, false, W><<<grid, block, row_smem<R>(H), s>>>(fb, g, p.tw_z, p.tw_post, scale);
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
  if (use_plane<R>(g)) {
    switch (g.ny) {
      case 16: set_plane_attr_ny<R, 16>(g.nz / 2); break;
      case 32: set_plane_attr_ny<R, 32>(g.nz / 2); break;
      case 64: set_plane_attr_ny<R, 64>(g.nz / 2); break;
      default: set_plane_attr_ny<R, 128>(g.nz / 2); break;
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
void fft_pass(const FFTPlan<R> &p, const FieldBatch<R> &fb, int pass, cudaStream_t s) {
  const bool plane = use_plane<R>(p.g);
  switch (pass) {
    case 0:  // z rows + y pencils, forward
      if (plane) {
        launch_plane(p, fb, false, s);
      } else {
        launch_rows(p, fb, false, s);
        launch_pencils(p, fb, 1, false, s);
      }
      break;
    case 1: launch_pencils(p, fb, 0, false, s); break;  // x pencils, forward
    case 2: launch_pencils(p, fb, 0, true, s); break;   // x pencils, inverse
    default:                                            // y pencils + z rows, inverse
      if (plane) {
        launch_plane(p, fb, true, s);
      } else {
        launch_herm_columns(p, fb, s);
        launch_pencils(p, fb, 1, true, s);
        launch_rows(p, fb, true, s);
      }
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
