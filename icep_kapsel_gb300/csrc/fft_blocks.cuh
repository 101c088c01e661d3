// fft_blocks.cuh -- device building blocks of the FFT kernels: in-register
// radix-8/4/2 DFTs, Stockham stages over shared-memory tiles, the real
// split/merge of z rows and the x-plane transform cores. Included by the FFT
// pass kernels (fft.cu) and the fused k-space operator (kop.cu).
//
// Every 1D transform is a Stockham autosort FFT with radix-8/4/2 stages held
// in registers (block_fft): a pencil of N complex values is split into N/8
// work items per stage, each one radix-8 (or two radix-4, four radix-2)
// butterflies; the items of all pencils a block owns are spread over its
// threads, and stages exchange data through padded shared-memory tiles
// (element e of pencil w at tile[e*sw + w], conflict-free). The inverse is
// conj(FFT(conj(x))), so only forward butterflies and twiddles exist.
#pragma once
#include "dfloat.cuh"
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
  const R h = sqrt_half<R>();
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
    const cplx<R> v = g.data[q + e * g.estride];
    // the four special pencils by their indices (no division per load):
    // kz = 0 at q = 0 and (NY/2) hnz, kz = NZ/2 at hnz - 1 and (NY/2) hnz + hnz - 1
    const long qh = (long)(ny / 2) * hnz;
    const bool kz0 = (q == 0 || q == qh), kzh = (q == hnz - 1 || q == qh + hnz - 1);
    if (kz0 || kzh) {
      if (e == 0 || e == nx / 2) return cplx<R>{v.x, R(0)};
      const bool kept = kz0 ? (e <= nx / 2) : (e > nx / 2);
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
  const R er = half_of(z.x + c.x), ei = half_of(z.y + c.y);
  const R orr = half_of(z.y - c.y), oi = half_of(c.x - z.x);
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

// ---- warp-local transforms --------------------------------------------------
// Shared tile with an XOR swizzle: element e of pencil w at
// t[e*sw + (w ^ ((e ^ (e >> 3)) & 15))], sw a multiple of 16. The lane groups
// of group_fft read elements 1 apart and write elements up to 8 apart within
// one pencil; the swizzle spreads both patterns over all banks.
__host__ __device__ __forceinline__ int swz(int e, int w, int sw) { return e * sw + (w ^ ((e ^ (e >> 3)) & 15)); }
template <typename R>
struct SmemX {
  cplx<R> *t;
  int sw;
  __device__ __forceinline__ cplx<R> load(int w, int e) const { return t[swz(e, w, sw)]; }
  __device__ __forceinline__ void store(int w, int e, cplx<R> v) const { t[swz(e, w, sw)] = v; }
};

// One Stockham stage of pencil w done by lane tl of its group of T = N/8
// lanes (the same butterflies as stage(), distributed over the group).
template <typename R, int N, int RAD, class Src, class Dst>
__device__ __forceinline__ void gstage(const Src &src, const Dst &dst, int w, int tl, int Ls,
                                       const cplx<R> *__restrict__ tws, bool conj_in, bool conj_out) {
  constexpr int T = N / 8;
  constexpr int NB = 8 / RAD;
#pragma unroll
  for (int m = 0; m < NB; m++) {
    const int jb = tl + T * m;
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

// Length-N transforms of NPEN pencils with every pencil on one lane group of
// T = N/8 lanes inside a warp, so that consecutive stages are ordered by
// __syncwarp alone. Groups take pencils in rounds that every lane runs (idle
// lanes included). First stage reads `in`, last writes `out`; intermediate
// stages alternate between tiles a and b (stride sw).
// Intermediate tiles are swizzled (SmemX); the groups that share a half-warp
// get pencils T apart, so a half-warp's accesses never collide.
// The caller synchronises the block around the call where other groups'
// pencils are read or written.
template <typename R, int N, int NPEN, class In, class Out>
__device__ __forceinline__ void group_fft(const In &in, const Out &out, cplx<R> *a, cplx<R> *b, int sw,
                                          const cplx<R> *tws, bool inverse) {
  constexpr int T = N / 8;
  static_assert(T >= 1 && T <= 32 && (32 % T) == 0, "a pencil's lane group must fit in a warp");
  const int lin = threadIdx.y * blockDim.x + threadIdx.x;
  const int ngroups = (blockDim.x * blockDim.y) / T;
  const int tl = lin % T;
  int w0;  // this group's pencil in round 0
  if (T >= 32) {
    w0 = lin / 32;
  } else {
    const int wi = lin >> 5, g = (lin & 31) / T;   // warp, group within the warp
    const int per = 16 / (T < 16 ? T : 16);        // groups per half-warp
    const int h = g / per, c = g - h * per;        // half-warp, position in it
    const int wpg = (T >= 2) ? T / 2 : 1;          // warps per 16 pencils
    w0 = (wi / wpg) * 16 + (wi % wpg) * 2 + c * T + h;
  }
  const int rounds = (NPEN + ngroups - 1) / ngroups;
  SmemX<R> ta{a, sw}, tb{b, sw};
  for (int r = 0; r < rounds; r++) {
    const int w = w0 + r * ngroups;
    const bool act = w < NPEN;
    int Ls = 1;
#pragma unroll
    for (int s = 0; s < Plan<N>::nstages; s++) {
      const int rad = Plan<N>::radix(s);
      const bool first = (s == 0), last = (s == Plan<N>::nstages - 1);
      const bool ci = first && inverse, co = last && inverse;
      const SmemX<R> &tsrc = (s & 1) ? tb : ta;
      const SmemX<R> &tdst = (s & 1) ? ta : tb;
      if (act) {
        if (first && last) {
          if (rad == 8) gstage<R, N, 8>(in, out, w, tl, Ls, tws, ci, co);
        } else if (first) {
          if (rad == 8) gstage<R, N, 8>(in, tb, w, tl, Ls, tws, ci, co);
          else if (rad == 4) gstage<R, N, 4>(in, tb, w, tl, Ls, tws, ci, co);
          else gstage<R, N, 2>(in, tb, w, tl, Ls, tws, ci, co);
        } else if (last) {
          if (rad == 8) gstage<R, N, 8>(tsrc, out, w, tl, Ls, tws, ci, co);
          else if (rad == 4) gstage<R, N, 4>(tsrc, out, w, tl, Ls, tws, ci, co);
          else gstage<R, N, 2>(tsrc, out, w, tl, Ls, tws, ci, co);
        } else {
          if (rad == 8) gstage<R, N, 8>(tsrc, tdst, w, tl, Ls, tws, ci, co);
          else if (rad == 4) gstage<R, N, 4>(tsrc, tdst, w, tl, Ls, tws, ci, co);
          else gstage<R, N, 2>(tsrc, tdst, w, tl, Ls, tws, ci, co);
        }
      }
      Ls *= rad;
      __syncwarp();
    }
  }
}

// ---- x-plane cores (one block per x-plane) -------------------------------
// smem: tw_y[NY] | tw_z[H] | post[H+1] | A | B, A/B of plane_tile() complex.
__host__ __device__ constexpr int plane_tile(int ny, int h) {
  return (h * (ny + 1) > ny * (h + 2)) ? h * (ny + 1) : ny * (h + 2);
}

// Forward core: the plane's NY real z rows, held as H-point complex rows in
// `rows` (element e of row j at rows[e*(NY+1) + j]), are transformed along z
// and y and written to the k-space plane `outp`. `other` is the second tile.
template <typename R, int NY, int H>
__device__ __forceinline__ void plane_fwd_core(cplx<R> *rows, cplx<R> *other, const cplx<R> *sty,
                                               const cplx<R> *stz, const cplx<R> *spost, const GPencils<R> &outp) {
  const int nthr = blockDim.x * blockDim.y, lin = threadIdx.y * blockDim.x + threadIdx.x;
  constexpr int rsw = NY + 1;
  // z transforms: rows -> (other, ...); with an even number of stages the result is in rows
  constexpr int zst = Plan<H>::nstages;
  cplx<R> *zres = (zst & 1) ? other : rows;
  cplx<R> *ybuf = (zst & 1) ? rows : other;
  block_fft<R, H, NY>(SmemT<R>{rows, rsw}, SmemT<R>{zres, rsw}, rows, other, rsw, stz, false);
  // split into the half spectrum, y-pencil layout: element j of pencil k at ybuf[j*ysw + k]
  constexpr int ysw = H + 2;
  for (int q = lin; q < NY * (H + 1); q += nthr) {
    const int j = q / (H + 1), k = q - j * (H + 1);
    const int k1 = (k == H) ? 0 : k, k2 = (k == 0) ? 0 : H - k;
    ybuf[j * ysw + k] = split_fwd(zres[k1 * rsw + j], cconj(zres[k2 * rsw + j]), spost[k]);
  }
  __syncthreads();
  // y transforms of the H+1 columns, last stage to global (coalesced over kz)
  cplx<R> *oth = (ybuf == rows) ? other : rows;
  block_fft<R, NY, H + 1>(SmemT<R>{ybuf, ysw}, outp, ybuf, oth, ysw, sty, false);
}

// Inverse core: the k-space plane, loaded into A in y-pencil layout
// (element j of column kz at A[j*(H+2) + kz]), is completed, transformed
// along y and z and left as H-point complex rows (element e of row j at
// result[e*(NY+1) + j], unscaled); returns the tile holding the result.
template <typename R, int NY, int H>
__device__ __forceinline__ cplx<R> *plane_inv_core(cplx<R> *A, cplx<R> *B, const cplx<R> *sty, const cplx<R> *stz,
                                                   const cplx<R> *spost) {
  const int nthr = blockDim.x * blockDim.y, lin = threadIdx.y * blockDim.x + threadIdx.x;
  constexpr int ysw = H + 2;
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
  return zres;
}

}  // namespace
}  // namespace icep
