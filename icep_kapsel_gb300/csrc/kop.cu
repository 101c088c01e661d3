// kop.cu -- see kop.cuh.
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "fft_blocks.cuh"
#include "kop.cuh"
#include "krylov.cuh"
#include "probe.cuh"

namespace icep {

namespace {

constexpr int KW = 16;  // x pencils per block
typedef cplx<float> cf;

__device__ __forceinline__ void kvec3(const Grid &g, int i, int j, int kz, float *k) {
  k[0] = g.wavef[0] * (float)kx_of(g, i);
  k[1] = g.wavef[1] * (float)ky_of(g, j);
  k[2] = g.wavef[2] * (float)kz;
}

// m(k) i k_D exp(i dx k_D / 2) p, m = -1/(eps_ref |k|^2), m(0) = 0
// the spectral preconditioner m(k) = -1/(eps_ref |k|^2), m(0) = 0
__device__ __forceinline__ float precond_m(const Grid &g, int i, int j, int kz, float ieps) {
  float k[3];
  kvec3(g, i, j, kz, k);
  const float k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
  return (k2 > 0.f) ? -ieps / k2 : 0.f;
}
// i k_D exp(i dx k_D / 2) p (p already multiplied by m(k))
template <int D>
__device__ __forceinline__ cf grad_mult(const Grid &g, int i, int j, int kz, cf p) {
  const float kd = g.wavef[D] * (float)((D == 0) ? kx_of(g, i) : (D == 1) ? ky_of(g, j) : kz);
  float cs, sn;
  shift_of(g, D, (D == 0) ? i : (D == 1) ? j : kz, cs, sn);
  const float gr = -kd * p.y, gi = kd * p.x;
  return cf{gr * cs - gi * sn, gr * sn + gi * cs};
}
// the x pass's source multiplier: the gradient's for D = 0, none for D < 0
// (the field M = m(k) p, whose y and z gradients the plane pass forms)
template <int D>
__device__ __forceinline__ cf xinv_mult(const Grid &g, int i, int j, int kz, cf p) {
  if constexpr (D < 0) return p;
  else return grad_mult<D>(g, i, j, kz, p);
}
// the gradient factor i k_D exp(i dx k_D/2) of D = 1 (y, idx = j) or D = 2
// (z, idx = kz); multiplying M by it commutes with the x transform
template <int D>
__device__ __forceinline__ cf grad_factor(const Grid &g, int idx) {
  const float kd = g.wavef[D] * (float)((D == 1) ? ky_of(g, idx) : idx);
  float cs, sn;
  shift_of(g, D, idx, cs, sn);
  return cf{-kd * sn, kd * cs};
}
// the divergence factor k_D exp(-i dx k_D/2) from the gradient factor (the
// overall i of the divergence is applied by the forward x pass)
__device__ __forceinline__ cf div_factor(cf c) { return cf{c.y, c.x}; }

// Block reduction of the threads' FP32 sums (s0, s1) times `scale` into
// partials[2*blockIdx.x + c]: FP32 within a warp, FP64 across the warps (one
// FP64 operation per warp instead of per thread: FP64 is scarce on GB300).
__device__ void block_partials(float s0, float s1, double scale, double *partials) {
  __shared__ double red[2][32];
  const int lin = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  const int lane = lin & 31, wid = lin >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
  }
  if (lane == 0) {
    red[0][wid] = (double)s0;
    red[1][wid] = (double)s1;
  }
  __syncthreads();
  if (lin < 2) {
    double v = 0.0;
    for (int w = 0; w < nthr / 32; w++) v += red[lin][w];
    partials[2 * blockIdx.x + lin] = v * scale;
  }
}

// block_partials, then the last block to finish sums every block's pair in a
// fixed order (lane b reads blocks b, b+32, ...; a shuffle tree combines the
// lanes) into finals[0..1] and re-arms the counter: the next kernel reads two
// numbers instead of all partials. Partials of other blocks are read through
// L2 (__ldcg) after the ticket, which follows each block's fence.
__device__ int block_partials_final(float s0, float s1, double scale, double *partials, double *finals,
                                    unsigned *counter) {
  block_partials(s0, s1, scale, partials);
  __shared__ int last;
  const int lin = threadIdx.y * blockDim.x + threadIdx.x;
  __threadfence();
  __syncthreads();
  if (lin == 0) last = (atomicAdd(counter, 1u) == gridDim.x * gridDim.y - 1) ? 1 : 0;
  __syncthreads();
  if (!last) return 0;
  __threadfence();
  if (lin < 64) {
    const int c = lin >> 5, lane = lin & 31;
    const int nb = (int)(gridDim.x * gridDim.y);
    double v = 0.0;
    for (int b = lane; b < nb; b += 32) v += __ldcg(partials + 2 * b + c);
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) finals[c] = v;
  }
  if (lin == 0) *counter = 0u;
  return 1;
}

// (j, kz) of pencils q0 .. q0 + W - 1 into shared arrays (synchronised by the caller)
template <int W>
__device__ __forceinline__ void pencil_coords(const Grid &g, int q0, int *pj, int *pkz) {
  const int lin = threadIdx.y * blockDim.x + threadIdx.x;
  if (lin < W) {
    const int q = q0 + lin;
    pj[lin] = q / g.hnz;
    pkz[lin] = q - (q / g.hnz) * g.hnz;
  }
}

__device__ __forceinline__ cf ldw(const float *a, long idx, int wt) {
  const float2 v = reinterpret_cast<const float2 *>(a)[idx];
  return cf{v.x, wt == 1 ? 0.f : v.y};
}

// First-stage source of the inverse x transforms: the updated vector times
// m(k), held in shared memory (`raw`, element e of pencil w at
// raw[e*sw + w]), times the x gradient multiplier (D = 0) or as it is
// (D < 0), with the i-direction half of the reference's Hermitian completion
// on the pencils (j, kz), j in {0, NY/2}, kz in {0, NZ/2} (as GPencilsXInv in
// the plain passes).
template <int D>
struct SrcGradXInv {
  const cf *raw;
  const int *pj, *pkz;  // (j, kz) of the block's pencils
  int sw, nvalid;
  Grid g;
  __device__ __forceinline__ cf load(int w, int e) const {
    if (w >= nvalid) return cf{0.f, 0.f};
    const int j = pj[w], kz = pkz[w];
    if ((j == 0 || j == g.ny / 2) && (kz == 0 || kz == g.hnz - 1)) {
      if (e == 0 || e == g.nx / 2) {
        const cf v = xinv_mult<D>(g, e, j, kz, cf{raw[e * sw + w].x, 0.f});
        return cf{v.x, 0.f};
      }
      const bool kept = (kz == 0) ? (e <= g.nx / 2) : (e > g.nx / 2);
      if (!kept) {
        const int m = g.nx - e;
        return cconj(xinv_mult<D>(g, m, j, kz, raw[m * sw + w]));
      }
    }
    return xinv_mult<D>(g, e, j, kz, raw[e * sw + w]);
  }
};

template <int N, int KWT, bool THREE>
__global__ void __launch_bounds__(512) k_kop_xinv(Grid g, int mode, float *vec, const float *r, const float *v,
                                                  float beta, float omega, double rho, const double *fin,
                                                  float ieps, float *w0, float *w1, float *w2, float *w3,
                                                  const cf *__restrict__ twx, const double *ks) {
  // device-side iteration state: beta, omega (P) and rho (S) from it
  if (ks) {
    beta = (float)__ldcg(ks + KS_BETA);
    omega = (float)__ldcg(ks + KS_OMEGA);
    rho = __ldcg(ks + KS_RHO);
    ieps = (float)__ldcg(ks + KS_IEPS);
  }
  extern __shared__ unsigned char smem_raw[];
  const int sw = KWT + 1;
  cf *tws = reinterpret_cast<cf *>(smem_raw);
  cf *raw = tws + N;
  cf *ta = raw + N * sw;
  cf *tb = ta + N * sw;
  const int nq = g.ny * g.hnz;
  const int q0 = blockIdx.x * KWT;
  const int nvalid = nq - q0 < KWT ? nq - q0 : KWT;
  const int lin = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  __shared__ int pj[KWT], pkz[KWT];
  load_table(tws, twx, N);
  pencil_coords<KWT>(g, q0, pj, pkz);
  __syncthreads();
  __shared__ float salpha;  // one FP64 division per block
  if (mode == KOP_S && lin == 0) salpha = (float)(rho / fin[0]);
  __syncthreads();
  const float alpha = (mode == KOP_S) ? salpha : 0.f;
  // vector update at the read modes of this block's pencils: xblock gives
  // KWT * N/8 threads, so every thread has XPT = 8 items; the loads of a batch
  // of XB items are issued together before any update is computed or stored
  static_assert(N / 8 <= 512 / KWT, "xblock(N) = KWT x N/8 threads");
  constexpr int XPT = 8, XB = 4;
  for (int u0 = 0; u0 < XPT; u0 += XB) {
    cf lr[XB], lv[XB], lp[XB];
#pragma unroll
    for (int u = 0; u < XB; u++) {
      const int it = lin + (u0 + u) * nthr;
      const int w = it % KWT, e = it / KWT;
      lr[u] = lv[u] = lp[u] = cf{0.f, 0.f};
      if (w >= nvalid) continue;
      const long idx = (long)e * nq + q0 + w;
      const int wt = read_weight(g, e, pj[w], pkz[w]);
      if (mode == KOP_NONE) {
        lp[u] = ldw(vec, idx, wt);
        continue;
      }
      lr[u] = ldw(r, idx, wt);
      if (mode != KOP_PC) lv[u] = ldw(v, idx, wt);
      if (mode == KOP_P || mode == KOP_PC) lp[u] = ldw(vec, idx, wt);
    }
#pragma unroll
    for (int u = 0; u < XB; u++) {
      const int it = lin + (u0 + u) * nthr;
      const int w = it % KWT, e = it / KWT;
      if (w >= nvalid) {
        raw[e * sw + w] = cf{0.f, 0.f};
        continue;
      }
      const int j = pj[w], kz = pkz[w];
      // raw holds the vector times the preconditioner m(k), once per mode for
      // the x gradient and M
      const float mk = precond_m(g, e, j, kz, ieps);
      cf nv;
      if (mode == KOP_NONE) {
        nv = lp[u];
      } else if (mode == KOP_P) {
        nv = cf{lr[u].x + beta * (lp[u].x - omega * lv[u].x), lr[u].y + beta * (lp[u].y - omega * lv[u].y)};
      } else if (mode == KOP_PC) {
        nv = cf{lr[u].x + beta * lp[u].x, lr[u].y + beta * lp[u].y};
      } else {
        nv = cf{lr[u].x - alpha * lv[u].x, lr[u].y - alpha * lv[u].y};
      }
      raw[e * sw + w] = cf{nv.x * mk, nv.y * mk};
      if (mode != KOP_NONE && read_weight(g, e, j, kz) > 0)
        reinterpret_cast<float2 *>(vec)[(long)e * nq + q0 + w] = make_float2(nv.x, nv.y);
    }
  }
  __syncthreads();
  // the x gradient into w0 and M = m(k) p into w1: the y and z gradient
  // multipliers depend on (j, kz) only, so the plane pass applies them to M;
  // with THREE (the split plane step, whose generic passes take no
  // factors) the y and z gradients themselves into w2 and w3
  block_fft<float, N, KWT>(SrcGradXInv<0>{raw, pj, pkz, sw, nvalid, g},
                          GPencils<float>{reinterpret_cast<cf *>(w0), (long)q0, 1, (long)nq, nvalid}, ta, tb, sw,
                          tws, true);
  if constexpr (THREE) {
    block_fft<float, N, KWT>(SrcGradXInv<1>{raw, pj, pkz, sw, nvalid, g},
                            GPencils<float>{reinterpret_cast<cf *>(w2), (long)q0, 1, (long)nq, nvalid}, ta, tb, sw,
                            tws, true);
    block_fft<float, N, KWT>(SrcGradXInv<2>{raw, pj, pkz, sw, nvalid, g},
                            GPencils<float>{reinterpret_cast<cf *>(w3), (long)q0, 1, (long)nq, nvalid}, ta, tb, sw,
                            tws, true);
  } else {
    block_fft<float, N, KWT>(SrcGradXInv<-1>{raw, pj, pkz, sw, nvalid, g},
                            GPencils<float>{reinterpret_cast<cf *>(w1), (long)q0, 1, (long)nq, nvalid}, ta, tb, sw,
                            tws, true);
  }
}

// Last-stage sink of the inverse z transforms: the real row values times the
// face permittivity, which carries the C2R scaling (FP32, rows of the x-plane).
struct MulSink {
  cf *t;
  int sw;
  const float *efp;  // eps_face_d of this x-plane (shared memory)
  int nzp;
  __device__ __forceinline__ void store(int w, int e, cf v) const {
    const float2 f = reinterpret_cast<const float2 *>(efp + w * nzp)[e];
    t[swz(e, w, sw)] = cf{v.x * f.x, v.y * f.y};
  }
};

// Row strides of the plane kernel's swizzled tiles (multiples of 16 complex
// values covering the pencil indices, see SmemX): the y layout holds columns
// 0..H-1 (the kz = NZ/2 column travels packed into column 0), the z layout
// rows 0..NY-1. A tile also holds one raw plane (NY x (H+1)) on arrival.
__host__ __device__ constexpr int kplane_ysw(int h) { return ((h + 15) / 16) * 16; }
__host__ __device__ constexpr int kplane_rsw(int ny) { return ((ny + 15) / 16) * 16; }
__host__ __device__ constexpr int kmax(int a, int b) { return a > b ? a : b; }
__host__ __device__ constexpr int kplane_tile(int ny, int h) {
  return kmax(kmax(h * kplane_rsw(ny), ny * kplane_ysw(h)), ny * (h + 1));
}
// bytes of the plane kernel's shared memory: eps_face plane (NY x NZ_ floats),
// two tiles, twiddles (NY + H + H+1), packed column, kz = NZ/2 column, 2 mbarriers
__host__ __device__ constexpr size_t kplane_smem(int ny, int h) {
  return (size_t)ny * (2 * h + 2) * sizeof(float) + 2 * (size_t)kplane_tile(ny, h) * sizeof(cf) +
         ((size_t)ny + h + (h + 1) + 2 * ny) * sizeof(cf) + 2 * sizeof(unsigned long long);
}

// ---- bulk asynchronous copies (1D TMA) with mbarrier completion ------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}
// global -> shared copy of `bytes` (multiple of 16, both addresses 16-byte aligned)
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}
__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Wait for phase `parity` of the mbarrier for at most `limit_ns` of
// %globaltimer time (a preempted kernel sees the copy complete when it
// resumes, so a time limit does not fire under load); false on timeout.
__device__ __forceinline__ bool mbar_wait_for(uint32_t mbar, uint32_t parity, unsigned long long limit_ns) {
  const unsigned long long t0 = globaltimer();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
    if (globaltimer() - t0 > limit_ns) return false;
  }
}
// Copy-arrival limit of the plane passes (a 66 KB copy lands in
// microseconds) and the short limit of the bounded-wait self-test.
constexpr unsigned long long KOP_WAIT_NS = 200ull * 1000 * 1000;
constexpr unsigned long long KOP_TEST_WAIT_NS = 50ull * 1000;

// First-stage source of the y transforms with the kz = 0 and kz = NZ/2
// columns packed into pencil 0 (p holds that pencil's elements).
struct SrcPacked {
  const cf *t;
  int sw;
  const cf *p;
  __device__ __forceinline__ cf load(int w, int e) const { return w == 0 ? p[e] : t[swz(e, w, sw)]; }
};

// One block per (x-plane, component): the plane's y/z inverse transform, the
// product with the face permittivity and the z/y forward transform. The raw
// k-space plane and the eps_face plane arrive by bulk asynchronous copies
// (the latter overlapping the y phase). Every 1D transform runs on one lane
// group of a warp (group_fft); the block synchronises only where a phase
// reads other groups' pencils (the two y <-> z re-layouts, the real
// merge/split and the global load/store). The kz = 0 and kz = NZ/2 columns
// are Hermitian in j on the way in and real in j on the way out, so they
// travel as one complex column (Z = X0 + i XH), leaving H y transforms.
template <int NY, int H>
__global__ void __launch_bounds__(1024) k_kop_plane(Grid g, float *w0, float *w1, float *w2, float *w3,
                                                    const float *ef0, const float *ef1, const float *ef2,
                                                    const cf *__restrict__ twy, const cf *__restrict__ twz,
                                                    const cf *__restrict__ post, int *err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int ysw = kplane_ysw(H), rsw = kplane_rsw(NY), TILE = kplane_tile(NY, H);
  constexpr int NZP = 2 * H + 2;
  float *efs = reinterpret_cast<float *>(smem_raw);  // eps_face_d of the plane, [j][NZ_]
  cf *A = reinterpret_cast<cf *>(efs + NY * NZP);
  cf *B = A + TILE;
  cf *sty = B + TILE;
  cf *stz = sty + NY;
  cf *spost = stz + H;
  cf *pk = spost + (H + 1);  // the packed column
  cf *colh = pk + NY;        // the kz = NZ/2 column as loaded
  unsigned long long *mb = reinterpret_cast<unsigned long long *>(colh + NY);
  const int i = blockIdx.x, d = blockIdx.y;
  const float *src = (d == 0) ? w0 : w1;
  float *dst = (d == 0) ? w0 : (d == 1) ? w2 : w3;
  const float *ef = (d == 0) ? ef0 : (d == 1) ? ef1 : ef2;
  const int nthr = blockDim.x * blockDim.y, lin = threadIdx.y * blockDim.x + threadIdx.x;
  const cf *cplane = reinterpret_cast<const cf *>(src) + (long)i * NY * (H + 1);
  cf *oplane = reinterpret_cast<cf *>(dst) + (long)i * NY * (H + 1);
  const float *efp = ef + (long)i * NY * NZP;
  constexpr uint32_t PLANE_BYTES = NY * (H + 1) * sizeof(cf), EF_BYTES = NY * NZP * sizeof(float);
  const uint32_t mb0 = smem_addr(&mb[0]), mb1 = smem_addr(&mb[1]);
  if (lin == 0) {
    mbar_init(mb0, 1);
    mbar_init(mb1, 1);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (lin == 0) {
    mbar_expect_tx(mb0, PLANE_BYTES);
    bulk_g2s(smem_addr(B), cplane, PLANE_BYTES, mb0);
    mbar_expect_tx(mb1, EF_BYTES);
    bulk_g2s(smem_addr(efs), efp, EF_BYTES, mb1);
  }
  load_table(sty, twy, NY);
  load_table(stz, twz, H);
  load_table(spost, post, H + 1);
  if (__syncthreads_or(!mbar_wait_for(mb0, 0, KOP_WAIT_NS))) {
    // a copy did not land: report it, let both copies finish before the
    // block's shared memory is released, and leave
    if (lin == 0) atomicExch(err, 1);
    mbar_wait_for(mb0, 0, KOP_WAIT_NS);
    mbar_wait_for(mb1, 0, KOP_WAIT_NS);
    return;
  }
  // raw plane [j][k] (in B) -> swizzled y layout (columns 0..H-1) + column H;
  // components 1 and 2 take their gradient factor here (before the
  // completion, as the x gradient's is taken before the x completion)
  for (int q = lin; q < NY * (H + 1); q += nthr) {
    const int j = q / (H + 1), k = q - j * (H + 1);
    cf v = B[q];
    if (d == 1) v = cmul(v, grad_factor<1>(g, j));
    else if (d == 2) v = cmul(v, grad_factor<2>(g, k));
    if (k < H) A[swz(j, k, ysw)] = v;
    else colh[j] = v;
  }
  __syncthreads();
  // the j-direction half of the Hermitian completion (kz = 0 keeps rows
  // 1..NY/2-1, kz = NZ/2 keeps rows NY/2+1..NY-1; rows 0, NY/2 are complete)
  // and the packing Z = X0 + i XH of the two completed columns
  for (int j = lin; j < NY; j += nthr) {
    const int m = (NY - j) & (NY - 1);
    const bool low = (j >= 1 && j < NY / 2), high = (j > NY / 2);
    const cf x0 = high ? cconj(A[swz(m, 0, ysw)]) : A[swz(j, 0, ysw)];
    const cf xh = low ? cconj(colh[m]) : colh[j];
    pk[j] = cf{x0.x - xh.y, x0.y + xh.x};
  }
  __syncthreads();
  // y inverse of the H columns (pencil 0 packed)
  constexpr int yst = Plan<NY>::nstages;
  cf *yres = (yst & 1) ? B : A;
  cf *zbuf = (yst & 1) ? A : B;
  group_fft<float, NY, H>(SrcPacked{A, ysw, pk}, SmemX<float>{yres, ysw}, A, B, ysw, sty, true);
  __syncthreads();
  // merge into H-point complex rows; column 0 holds x0 + i xh (both real)
  for (int q = lin; q < NY * H; q += nthr) {
    const int j = q / H, k = q - j * H;
    cf x, c;
    if (k == 0) {
      const cf z = yres[swz(j, 0, ysw)];
      x = cf{z.x, 0.f};
      c = cf{z.y, 0.f};
    } else {
      x = yres[swz(j, k, ysw)];
      c = yres[swz(j, H - k, ysw)];
    }
    zbuf[swz(k, j, rsw)] = merge_inv(x, cconj(c), spost[k]);
  }
  if (__syncthreads_or(!mbar_wait_for(mb1, 0, KOP_WAIT_NS))) {
    if (lin == 0) atomicExch(err, 1);
    mbar_wait_for(mb1, 0, KOP_WAIT_NS);
    return;
  }
  // z inverse, times the scaled face permittivity, z forward: row j stays on
  // the same lane group throughout, so no block synchronisation in between
  constexpr int zst = Plan<H>::nstages;
  cf *other = (zbuf == A) ? B : A;
  cf *rows = (zst & 1) ? other : zbuf;
  MulSink ms{rows, rsw, efs, NZP};
  group_fft<float, H, NY>(SmemX<float>{zbuf, rsw}, ms, zbuf, other, rsw, stz, true);
  cf *rother = (rows == A) ? B : A;
  cf *zf = (zst & 1) ? rother : rows;
  group_fft<float, H, NY>(SmemX<float>{rows, rsw}, SmemX<float>{zf, rsw}, rows, rother, rsw, stz, false);
  __syncthreads();
  // split into the half spectrum (y-pencil layout); the real kz = 0 and
  // kz = NZ/2 values are packed into column 0
  cf *ybuf = (zf == A) ? B : A;
  for (int q = lin; q < NY * H; q += nthr) {
    const int j = q / H, k = q - j * H;
    if (k == 0) {
      const cf z0 = zf[swz(0, j, rsw)], c0 = cconj(z0);
      const float x0 = split_fwd(z0, c0, spost[0]).x, xh = split_fwd(z0, c0, spost[H]).x;
      ybuf[swz(j, 0, ysw)] = cf{x0, xh};
    } else {
      ybuf[swz(j, k, ysw)] = split_fwd(zf[swz(k, j, rsw)], cconj(zf[swz(H - k, j, rsw)]), spost[k]);
    }
  }
  __syncthreads();
  // y forward of the H columns, then the unpacking of column 0 and a
  // coalesced store
  cf *yo = (ybuf == A) ? B : A;
  cf *yout = (yst & 1) ? yo : ybuf;
  group_fft<float, NY, H>(SmemX<float>{ybuf, ysw}, SmemX<float>{yout, ysw}, ybuf, yo, ysw, sty, false);
  __syncthreads();
  for (int q = lin; q < NY * (H + 1); q += nthr) {
    const int j = q / (H + 1), k = q - j * (H + 1);
    cf v;
    if (k == 0 || k == H) {
      const cf z = yout[swz(j, 0, ysw)], zm = cconj(yout[swz((NY - j) & (NY - 1), 0, ysw)]);
      v = (k == 0) ? cf{0.5f * (z.x + zm.x), 0.5f * (z.y + zm.y)} : cf{0.5f * (z.y - zm.y), -0.5f * (z.x - zm.x)};
    } else {
      v = yout[swz(j, k, ysw)];
    }
    // components 1 and 2: their divergence factor
    if (d == 1) v = cmul(v, div_factor(grad_factor<1>(g, j)));
    else if (d == 2) v = cmul(v, div_factor(grad_factor<2>(g, k)));
    oplane[q] = v;
  }
}

// ---- register-resident plane pass -------------------------------------------
//
// The same transform as k_kop_plane with the 1D transforms held in registers:
// a length-N DFT (N = T P) runs on T threads, thread t holding x[t + T m] for
// m < P. Step 1 is a P-point DFT over m in registers and the twiddle
// w_N^(t q1); one exchange through a shared region hands thread t' the T
// values b[tau][q1] for q1 = t' + T s (s < P/T); step 2 is a T-point DFT over
// tau, which leaves X[q1 + P q2] in register r = s + (P/T) q2, i.e. thread t'
// holds X[t' + T r]: the output has the input's distribution, so an inverse
// transform, the permittivity product and a forward transform chain with no
// re-layout in between. A plane costs one shared-memory exchange per 1D
// transform instead of one per radix stage.

constexpr float KC1 = 0.92387953251128675613f;  // cos(pi/8)
constexpr float KS1 = 0.38268343236508977173f;  // sin(pi/8)
constexpr float KH = 0.70710678118654752440f;   // sqrt(1/2)

// 16-point forward DFT in registers, natural order: 4 x 4 with the twiddles
// w_16^(n1 k1) between the two radix-4 layers.
__device__ __forceinline__ void dft16(cf *x) {
  cf u[4][4];
#pragma unroll
  for (int n1 = 0; n1 < 4; n1++) {
    cf v[4] = {x[n1], x[n1 + 4], x[n1 + 8], x[n1 + 12]};
    dft4(v);
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) u[n1][k1] = v[k1];
  }
  const cf w1{KC1, -KS1}, w2{KH, -KH}, w3{KS1, -KC1}, w6{-KH, -KH}, w9{-KC1, KS1};
  u[1][1] = cmul(u[1][1], w1);
  u[1][2] = cmul(u[1][2], w2);
  u[1][3] = cmul(u[1][3], w3);
  u[2][1] = cmul(u[2][1], w2);
  u[2][2] = mul_mi(u[2][2]);
  u[2][3] = cmul(u[2][3], w6);
  u[3][1] = cmul(u[3][1], w3);
  u[3][2] = cmul(u[3][2], w6);
  u[3][3] = cmul(u[3][3], w9);
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) {
    cf v[4] = {u[0][k1], u[1][k1], u[2][k1], u[3][k1]};
    dft4(v);
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) x[k1 + 4 * k2] = v[k2];
  }
}
template <int P>
__device__ __forceinline__ void dftp(cf *x) {
  static_assert(P == 4 || P == 8 || P == 16, "register DFT length");
  if constexpr (P == 16) dft16(x);
  else if constexpr (P == 8) dft8(x);
  else dft4(x);
}

// Position of b[tau][q1] in an exchange region of T*P values: T per q1, the
// thread index XOR-swizzled so that both the writes (fixed q1) and the reads
// (fixed tau, q1 = t' + T s) of a half-warp hit distinct banks; `par` is bit
// 3 of the region index (regions 8 apart share a half-warp for T = 8).
template <int T>
__device__ __forceinline__ int xpos(int q1, int tau, int par) {
  if constexpr (T == 8) return 8 * q1 + (tau ^ ((q1 >> 1) & 3) ^ (par << 2));
  else return 4 * q1 + (tau ^ (q1 & 3));
}

// Length-(T P) DFT of the thread's P registers (see above): forward, or the
// inverse as conj(DFT(conj x)). `reg` is the transform's exchange region,
// `tw` the table w_N^m, m < N. The caller orders reuse of `reg` around it.
template <int T, int P>
__device__ __forceinline__ void reg_dft(cf *x, int t, cf *reg, int par, const cf *tw, bool inverse) {
  static_assert(P >= T, "each thread takes P/T of the T-point DFTs");
  if (inverse) {
#pragma unroll
    for (int m = 0; m < P; m++) x[m] = cconj(x[m]);
  }
  dftp<P>(x);
#pragma unroll
  for (int q1 = 1; q1 < P; q1++) x[q1] = cmul(x[q1], tw[t * q1]);
#pragma unroll
  for (int q1 = 0; q1 < P; q1++) reg[xpos<T>(q1, t, par)] = x[q1];
  __syncwarp();
  constexpr int S = P / T;
#pragma unroll
  for (int s = 0; s < S; s++) {
    cf c[T];
    const int q1 = t + T * s;
#pragma unroll
    for (int tau = 0; tau < T; tau++) c[tau] = reg[xpos<T>(q1, tau, par)];
    dftp<T>(c);
#pragma unroll
    for (int q2 = 0; q2 < T; q2++) x[s + S * q2] = inverse ? cconj(c[q2]) : c[q2];
  }
}

// shared -> global bulk copy of `bytes` from this CTA (16-byte aligned
// addresses, size a multiple of 16) as the CTA's last step: waited for until
// the shared memory has been read (the writes complete with the grid), so
// the CTA's slot is released without waiting for them
__device__ __forceinline__ void bulk_s2g_wait(void *dst, uint32_t src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// Thread shapes of the register plane pass: y transforms on TY = 8 threads
// (PY = NY/8 values each) for the H columns; z transforms on TZ threads for
// the NY rows, RZ rows per thread in turn.
template <int NY, int H>
struct RPlane {
  static constexpr int TY = 8, PY = NY / 8;
  static constexpr int TZ = (H >= 64) ? 8 : 4, PZ = H / TZ;
  static constexpr int NT = H * TY;
  static constexpr int RZ = NY * TZ / NT;
  static constexpr int BUF = NY * (H + 1);  // complex values: the plane, [j][kz]
  static constexpr int ER = NY < 64 ? NY : 64;  // rows of the z phase's first round (0..ER-1)
  static constexpr int EBUF = ER * (H + 1);     // their face permittivities, float pairs
  static_assert(PY >= TY && PZ >= TZ && RZ >= 1 && RZ <= 2 && NY * TZ == RZ * NT, "register plane shape");
  static_assert(H <= NY, "the y exchange regions fit in the plane buffer");
};
template <int NY, int H>
__host__ __device__ constexpr size_t rplane_smem() {
  return ((size_t)RPlane<NY, H>::BUF + RPlane<NY, H>::EBUF + NY + H + (H + 1) + (NY + 1)) * sizeof(cf) +
         2 * sizeof(unsigned long long);
}

// Row j of the z phase for warp w, lane group jr, round p: rows of a
// half-warp 8 (TZ = 8) or 4 (TZ = 4) apart, which keeps the row-major tile
// accesses conflict-free.
template <int TZ>
__device__ __forceinline__ int rplane_row(int w, int jr, int p) {
  if constexpr (TZ == 8) return (w & 7) + 8 * jr + 32 * (w >> 3) + 64 * p;
  else return (w & 3) + 4 * jr + 32 * (w >> 2) + 64 * p;
}

// One block per (x-plane, component), H*8 threads. Component 0 transforms
// w0 (the x gradient) in place; components 1 and 2 read M (w1), take the y or
// z gradient factor on the way in and the divergence factor on the way out,
// and write w2 and w3. The plane arrives by one
// bulk copy into `buf` ([j][kz], row stride H+1) and leaves by one. y phase:
// thread (column k, t) holds rows t + 8m of its column (column 0 carries
// the packed kz = 0 and kz = NZ/2 columns after their Hermitian completion
// in j); z phase: thread (row j, tz) holds elements tz + TZ m of the merged
// H-point complex row, which after the inverse are the real row's values,
// multiplied by the face permittivity (read from global memory
// straight into registers) and transformed forward in place; the y forward
// transform reads the split half spectrum. `test_wait` (the bounded-wait
// self-test): no copy is issued and the wait runs out, which must reach the
// host through `err`.
template <int NY, int H>
__global__ void __launch_bounds__(H * 8, (H >= 64) ? 2 : 4)
    k_kop_plane_r(Grid g, float *w0, float *w1, float *w2, float *w3, const float *ef0, const float *ef1,
                  const float *ef2, const cf *__restrict__ twy, const cf *__restrict__ twz,
                  const cf *__restrict__ post, int *err, int test_wait) {
  using S = RPlane<NY, H>;
  constexpr int TY = S::TY, PY = S::PY, TZ = S::TZ, PZ = S::PZ, RS = H + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cf *buf = reinterpret_cast<cf *>(smem_raw);
  float2 *estage = reinterpret_cast<float2 *>(buf + S::BUF);  // eps_face rows 0..ER-1
  cf *sty = reinterpret_cast<cf *>(estage + S::EBUF);
  cf *stz = sty + NY;
  cf *spost = stz + H;
  cf *sfac = spost + H + 1;  // gradient factors: of row j (d = 1) or column kz (d = 2)
  unsigned long long *mb = reinterpret_cast<unsigned long long *>(sfac + NY + 1);
  const int i = blockIdx.x, d = blockIdx.y;
  const float *src = (d == 0) ? w0 : w1;
  float *dst = (d == 0) ? w0 : (d == 1) ? w2 : w3;
  const float *ef = (d == 0) ? ef0 : (d == 1) ? ef1 : ef2;
  const cf *cplane = reinterpret_cast<const cf *>(src) + (long)i * S::BUF;
  cf *oplane = reinterpret_cast<cf *>(dst) + (long)i * S::BUF;
  const float2 *efp = reinterpret_cast<const float2 *>(ef) + (long)i * S::BUF;  // [j][NZ_] floats as float2
  const int lin = threadIdx.x, lane = lin & 31, w = lin >> 5;
  constexpr uint32_t BYTES = S::BUF * sizeof(cf), EBYTES = S::EBUF * sizeof(float2);
  const uint32_t mb0 = smem_addr(&mb[0]), mb1 = smem_addr(&mb[1]);
  if (lin == 0) {
    mbar_init(mb0, 1);
    mbar_init(mb1, 1);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (lin == 0) {
    if (test_wait) {
      mbar_expect_tx(mb0, 16);  // transactions that nothing will complete
      mbar_expect_tx(mb1, 16);
    } else {
      mbar_expect_tx(mb0, BYTES);
      bulk_g2s(smem_addr(buf), cplane, BYTES, mb0);
      // the face permittivities of the z phase's first round of rows, which
      // land while the y transforms run
      mbar_expect_tx(mb1, EBYTES);
      bulk_g2s(smem_addr(estage), efp, EBYTES, mb1);
    }
  }
  // the rows of the second round go to L2 meanwhile (one 128-byte line per thread)
  if (S::RZ > 1 && !test_wait) {
    constexpr int LINES = (NY - S::ER) * (H + 1) * (int)sizeof(float2) / 128;
    for (int q = lin; q < LINES; q += S::NT)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(reinterpret_cast<const char *>(efp + S::EBUF) + 128 * q));
  }
  for (int q = lin; q < NY; q += S::NT) sty[q] = twy[q];
  for (int q = lin; q < H; q += S::NT) stz[q] = twz[q];
  for (int q = lin; q <= H; q += S::NT) spost[q] = post[q];
  if (d == 1)
    for (int q = lin; q < NY; q += S::NT) sfac[q] = grad_factor<1>(g, q);
  else if (d == 2)
    for (int q = lin; q <= H; q += S::NT) sfac[q] = grad_factor<2>(g, q);
  const unsigned long long lim = test_wait ? KOP_TEST_WAIT_NS : KOP_WAIT_NS;
  if (__syncthreads_or(!mbar_wait_for(mb0, 0, lim))) {
    // a copy did not land: report it, let copies still in flight finish
    // before the block's shared memory is released, and leave
    if (lin == 0) atomicExch(err, 1);
    if (!test_wait) {
      mbar_wait_for(mb0, 0, KOP_WAIT_NS);
      mbar_wait_for(mb1, 0, KOP_WAIT_NS);
    }
    return;
  }
  // ---- y inverse: thread (column k, t), rows t + 8m
  const int t = lane & 7, kc = lane >> 3;
  const int k = (w & 7) + 8 * kc + 32 * (w >> 3);
  const int par = (k >> 3) & 1;
  cf a[PY];
  // components 1 and 2: the gradient factor of the element's row or column,
  // taken before the completion (as the x gradient's before the x completion)
  if (k == 0) {
    // the j-direction half of the Hermitian completion of the kz = 0 and
    // kz = NZ/2 columns (kz = 0 keeps rows 1..NY/2-1, kz = NZ/2 keeps rows
    // NY/2+1..NY-1; rows 0 and NY/2 are used as they are), packed as
    // Z = X0 + i XH
#pragma unroll
    for (int m = 0; m < PY; m++) {
      const int j = t + 8 * m, jm = (NY - j) & (NY - 1);
      const bool low = (j >= 1 && j < NY / 2), high = (j > NY / 2);
      const int j0 = high ? jm : j, jh = low ? jm : j;
      cf x0 = buf[j0 * RS], xh = buf[jh * RS + H];
      if (d == 1) {
        x0 = cmul(x0, sfac[j0]);
        xh = cmul(xh, sfac[jh]);
      } else if (d == 2) {
        x0 = cmul(x0, sfac[0]);
        xh = cmul(xh, sfac[H]);
      }
      if (high) x0 = cconj(x0);
      if (low) xh = cconj(xh);
      a[m] = cf{x0.x - xh.y, x0.y + xh.x};
    }
  } else if (d == 1) {
#pragma unroll
    for (int m = 0; m < PY; m++) a[m] = cmul(buf[(t + 8 * m) * RS + k], sfac[t + 8 * m]);
  } else if (d == 2) {
    const cf fk = sfac[k];
#pragma unroll
    for (int m = 0; m < PY; m++) a[m] = cmul(buf[(t + 8 * m) * RS + k], fk);
  } else {
#pragma unroll
    for (int m = 0; m < PY; m++) a[m] = buf[(t + 8 * m) * RS + k];
  }
  __syncthreads();  // the plane is in registers: buf becomes exchange space
  reg_dft<TY, PY>(a, t, buf + k * (NY + 1), par, sty, true);
  __syncthreads();  // every column's exchange is read
#pragma unroll
  for (int r = 0; r < PY; r++) buf[(t + 8 * r) * RS + k] = a[r];
  if (__syncthreads_or(!mbar_wait_for(mb1, 0, KOP_WAIT_NS))) {
    if (lin == 0) atomicExch(err, 1);
    mbar_wait_for(mb1, 0, KOP_WAIT_NS);
    return;
  }
  // ---- z: merge, inverse, times the face permittivity (which carries the
  // inverse transform's 1/N), forward
  {
    const int tz = lane & (TZ - 1), jr = lane / TZ;
    // second-round permittivities from L2 into registers, in flight while
    // the first round runs on the staged ones
    float2 enext[PZ];
    if (S::RZ > 1) {
      const int j1 = rplane_row<TZ>(w, jr, 1);
#pragma unroll
      for (int m = 0; m < PZ; m++) enext[m] = __ldg(efp + j1 * RS + tz + TZ * m);
    }
#pragma unroll
    for (int p = 0; p < S::RZ; p++) {
      const int j = rplane_row<TZ>(w, jr, p);
      cf *row = buf + j * RS;
      cf z[PZ];
#pragma unroll
      for (int m = 0; m < PZ; m++) {
        const int n = tz + TZ * m;
        cf x, c;
        if (n == 0) {  // column 0 holds x0 + i xh, both real
          const cf zz = row[0];
          x = cf{zz.x, 0.f};
          c = cf{zz.y, 0.f};
        } else {
          x = row[n];
          c = row[H - n];
        }
        z[m] = merge_inv(x, cconj(c), spost[n]);
      }
      __syncwarp();  // the row's values are in registers: its storage becomes exchange space
      const int rpar = (j >> 3) & 1;
      reg_dft<TZ, PZ>(z, tz, row, rpar, stz, true);
#pragma unroll
      for (int m = 0; m < PZ; m++) {
        // first round: the staged rows, read only now; second: the registers
        const float2 e = (p == 0) ? estage[j * RS + tz + TZ * m] : enext[m];
        z[m] = cf{z[m].x * e.x, z[m].y * e.y};
      }
      __syncwarp();
      reg_dft<TZ, PZ>(z, tz, row, rpar, stz, false);
      __syncwarp();
#pragma unroll
      for (int m = 0; m < PZ; m++) row[tz + TZ * m] = z[m];
    }
  }
  __syncthreads();
  // ---- y forward of the split half spectrum (column 0: the real kz = 0 and
  // kz = NZ/2 values packed)
  if (k == 0) {
#pragma unroll
    for (int m = 0; m < PY; m++) {
      const cf z0 = buf[(t + 8 * m) * RS], c0 = cconj(z0);
      a[m] = cf{split_fwd(z0, c0, spost[0]).x, split_fwd(z0, c0, spost[H]).x};
    }
  } else {
#pragma unroll
    for (int m = 0; m < PY; m++) {
      const int j = t + 8 * m;
      a[m] = split_fwd(buf[j * RS + k], cconj(buf[j * RS + H - k]), spost[k]);
    }
  }
  __syncthreads();
  reg_dft<TY, PY>(a, t, buf + k * (NY + 1), par, sty, false);
  __syncthreads();
  // unpacking of column 0 (partner row NY - j: lane (8 - t) & 7 of the same
  // group, register PY-1-r; row 8r of lane 0 pairs with its own register
  // (PY - r) mod PY), then the plane to buf in its global layout
  if (w == 0) {
#pragma unroll
    for (int r = 0; r < PY; r++) {
      const int src = (lane & ~7) | ((8 - t) & 7);
      cf zm{__shfl_sync(0xffffffffu, a[PY - 1 - r].x, src), __shfl_sync(0xffffffffu, a[PY - 1 - r].y, src)};
      if (t == 0) zm = a[(PY - r) & (PY - 1)];
      if (k == 0) {
        const cf z = a[r], zc = cconj(zm);
        const int j = t + 8 * r;
        cf v0{0.5f * (z.x + zc.x), 0.5f * (z.y + zc.y)};
        cf vh{0.5f * (z.y - zc.y), -0.5f * (z.x - zc.x)};
        if (d == 1) {
          const cf f = div_factor(sfac[j]);
          v0 = cmul(v0, f);
          vh = cmul(vh, f);
        } else if (d == 2) {
          v0 = cmul(v0, div_factor(sfac[0]));
          vh = cmul(vh, div_factor(sfac[H]));
        }
        buf[j * RS] = v0;
        buf[j * RS + H] = vh;
      }
    }
  }
  // components 1 and 2: the divergence factor
  if (k != 0 && d == 1) {
#pragma unroll
    for (int r = 0; r < PY; r++) buf[(t + 8 * r) * RS + k] = cmul(a[r], div_factor(sfac[t + 8 * r]));
  } else if (k != 0 && d == 2) {
    const cf fk = div_factor(sfac[k]);
#pragma unroll
    for (int r = 0; r < PY; r++) buf[(t + 8 * r) * RS + k] = cmul(a[r], fk);
  } else if (k != 0) {
#pragma unroll
    for (int r = 0; r < PY; r++) buf[(t + 8 * r) * RS + k] = a[r];
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  if (lin == 0) bulk_s2g_wait(oplane, smem_addr(buf), BYTES);
}

// ---- register-resident plane passes of the plain 3D transforms -----------
//
// The two halves of k_kop_plane_r as the plane pass of the ordinary FP32
// transforms (fft.cuh): C2R (y inverse with the j-direction half of the
// Hermitian completion, then the z rows merged and inverse-transformed to the
// real row, scaled) and R2C (z rows forward, then the real split and the y
// forward). One block per (x-plane, field of the batch); the plane arrives by
// one bulk copy and leaves by one (a real plane of NY rows of NZ+2 floats has
// the byte size of the half-spectrum plane). A copy that does not land within
// the wait limit sets *err (checked by the host as for the fused passes).

// field f of a batch with constant indices (no local copy of the parameter)
__device__ __forceinline__ float *batch_field(const FieldBatch<float> &fb, int f) {
  float *q = fb.p[0];
#pragma unroll
  for (int c = 1; c < 5; c++)
    if (f == c) q = fb.p[c];
  return q;
}

template <int NY, int H>
__global__ void __launch_bounds__(H * 8, (H >= 64) ? 2 : 4)
    k_plane_c2r_r(FieldBatch<float> fb, const cf *__restrict__ twy, const cf *__restrict__ twz,
                  const cf *__restrict__ post, float scale, int *err) {
  using S = RPlane<NY, H>;
  constexpr int TY = S::TY, PY = S::PY, TZ = S::TZ, PZ = S::PZ, RS = H + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cf *buf = reinterpret_cast<cf *>(smem_raw);
  cf *sty = buf + S::BUF;
  cf *stz = sty + NY;
  cf *spost = stz + H;
  unsigned long long *mb = reinterpret_cast<unsigned long long *>(spost + H + 1);
  const int i = blockIdx.x;
  cf *cplane = reinterpret_cast<cf *>(batch_field(fb, blockIdx.y)) + (long)i * S::BUF;
  const int lin = threadIdx.x, lane = lin & 31, w = lin >> 5;
  constexpr uint32_t BYTES = S::BUF * sizeof(cf);
  const uint32_t mb0 = smem_addr(&mb[0]);
  if (lin == 0) {
    mbar_init(mb0, 1);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (lin == 0) {
    mbar_expect_tx(mb0, BYTES);
    bulk_g2s(smem_addr(buf), cplane, BYTES, mb0);
  }
  for (int q = lin; q < NY; q += S::NT) sty[q] = twy[q];
  for (int q = lin; q < H; q += S::NT) stz[q] = twz[q];
  for (int q = lin; q <= H; q += S::NT) spost[q] = post[q];
  if (__syncthreads_or(!mbar_wait_for(mb0, 0, KOP_WAIT_NS))) {
    if (lin == 0) atomicExch(err, 1);
    mbar_wait_for(mb0, 0, KOP_WAIT_NS);
    return;
  }
  // ---- y inverse: thread (column k, t), rows t + 8m (as in k_kop_plane_r)
  const int t = lane & 7, kc = lane >> 3;
  const int k = (w & 7) + 8 * kc + 32 * (w >> 3);
  const int par = (k >> 3) & 1;
  cf a[PY];
  if (k == 0) {
#pragma unroll
    for (int m = 0; m < PY; m++) {
      const int j = t + 8 * m, jm = (NY - j) & (NY - 1);
      const bool low = (j >= 1 && j < NY / 2), high = (j > NY / 2);
      const cf x0 = high ? cconj(buf[jm * RS]) : buf[j * RS];
      const cf xh = low ? cconj(buf[jm * RS + H]) : buf[j * RS + H];
      a[m] = cf{x0.x - xh.y, x0.y + xh.x};
    }
  } else {
#pragma unroll
    for (int m = 0; m < PY; m++) a[m] = buf[(t + 8 * m) * RS + k];
  }
  __syncthreads();
  reg_dft<TY, PY>(a, t, buf + k * (NY + 1), par, sty, true);
  __syncthreads();
#pragma unroll
  for (int r = 0; r < PY; r++) buf[(t + 8 * r) * RS + k] = a[r];
  __syncthreads();
  // ---- z: merge and inverse to the real row, scaled; its padding zeroed
  {
    const int tz = lane & (TZ - 1), jr = lane / TZ;
#pragma unroll
    for (int p = 0; p < S::RZ; p++) {
      const int j = rplane_row<TZ>(w, jr, p);
      cf *row = buf + j * RS;
      cf z[PZ];
#pragma unroll
      for (int m = 0; m < PZ; m++) {
        const int n = tz + TZ * m;
        cf x, c;
        if (n == 0) {
          const cf zz = row[0];
          x = cf{zz.x, 0.f};
          c = cf{zz.y, 0.f};
        } else {
          x = row[n];
          c = row[H - n];
        }
        z[m] = merge_inv(x, cconj(c), spost[n]);
      }
      __syncwarp();
      reg_dft<TZ, PZ>(z, tz, row, (j >> 3) & 1, stz, true);
      __syncwarp();
#pragma unroll
      for (int m = 0; m < PZ; m++) row[tz + TZ * m] = cf{z[m].x * scale, z[m].y * scale};
      if (tz == 0) row[H] = cf{0.f, 0.f};
    }
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  if (lin == 0) bulk_s2g_wait(cplane, smem_addr(buf), BYTES);
}

template <int NY, int H>
__global__ void __launch_bounds__(H * 8, (H >= 64) ? 2 : 4)
    k_plane_r2c_r(FieldBatch<float> fb, const cf *__restrict__ twy, const cf *__restrict__ twz,
                  const cf *__restrict__ post, int *err) {
  using S = RPlane<NY, H>;
  constexpr int TY = S::TY, PY = S::PY, TZ = S::TZ, PZ = S::PZ, RS = H + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cf *buf = reinterpret_cast<cf *>(smem_raw);
  cf *sty = buf + S::BUF;
  cf *stz = sty + NY;
  cf *spost = stz + H;
  unsigned long long *mb = reinterpret_cast<unsigned long long *>(spost + H + 1);
  const int i = blockIdx.x;
  cf *cplane = reinterpret_cast<cf *>(batch_field(fb, blockIdx.y)) + (long)i * S::BUF;
  const int lin = threadIdx.x, lane = lin & 31, w = lin >> 5;
  constexpr uint32_t BYTES = S::BUF * sizeof(cf);
  const uint32_t mb0 = smem_addr(&mb[0]);
  if (lin == 0) {
    mbar_init(mb0, 1);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (lin == 0) {
    mbar_expect_tx(mb0, BYTES);
    bulk_g2s(smem_addr(buf), cplane, BYTES, mb0);
  }
  for (int q = lin; q < NY; q += S::NT) sty[q] = twy[q];
  for (int q = lin; q < H; q += S::NT) stz[q] = twz[q];
  for (int q = lin; q <= H; q += S::NT) spost[q] = post[q];
  if (__syncthreads_or(!mbar_wait_for(mb0, 0, KOP_WAIT_NS))) {
    if (lin == 0) atomicExch(err, 1);
    mbar_wait_for(mb0, 0, KOP_WAIT_NS);
    return;
  }
  // ---- z forward of each real row as an H-point complex row, in place
  {
    const int tz = lane & (TZ - 1), jr = lane / TZ;
#pragma unroll
    for (int p = 0; p < S::RZ; p++) {
      const int j = rplane_row<TZ>(w, jr, p);
      cf *row = buf + j * RS;
      cf z[PZ];
#pragma unroll
      for (int m = 0; m < PZ; m++) z[m] = row[tz + TZ * m];
      __syncwarp();
      reg_dft<TZ, PZ>(z, tz, row, (j >> 3) & 1, stz, false);
      __syncwarp();
#pragma unroll
      for (int m = 0; m < PZ; m++) row[tz + TZ * m] = z[m];
    }
  }
  __syncthreads();
  // ---- y forward of the split half spectrum (as in k_kop_plane_r)
  const int t = lane & 7, kc = lane >> 3;
  const int k = (w & 7) + 8 * kc + 32 * (w >> 3);
  const int par = (k >> 3) & 1;
  cf a[PY];
  if (k == 0) {
#pragma unroll
    for (int m = 0; m < PY; m++) {
      const cf z0 = buf[(t + 8 * m) * RS], c0 = cconj(z0);
      a[m] = cf{split_fwd(z0, c0, spost[0]).x, split_fwd(z0, c0, spost[H]).x};
    }
  } else {
#pragma unroll
    for (int m = 0; m < PY; m++) {
      const int j = t + 8 * m;
      a[m] = split_fwd(buf[j * RS + k], cconj(buf[j * RS + H - k]), spost[k]);
    }
  }
  __syncthreads();
  reg_dft<TY, PY>(a, t, buf + k * (NY + 1), par, sty, false);
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int r = 0; r < PY; r++) {
      const int src = (lane & ~7) | ((8 - t) & 7);
      cf zm{__shfl_sync(0xffffffffu, a[PY - 1 - r].x, src), __shfl_sync(0xffffffffu, a[PY - 1 - r].y, src)};
      if (t == 0) zm = a[(PY - r) & (PY - 1)];
      if (k == 0) {
        const cf z = a[r], zc = cconj(zm);
        const int j = t + 8 * r;
        buf[j * RS] = cf{0.5f * (z.x + zc.x), 0.5f * (z.y + zc.y)};
        buf[j * RS + H] = cf{0.5f * (z.y - zc.y), -0.5f * (z.x - zc.x)};
      }
    }
  }
  if (k != 0) {
#pragma unroll
    for (int r = 0; r < PY; r++) buf[(t + 8 * r) * RS + k] = a[r];
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  if (lin == 0) bulk_s2g_wait(cplane, smem_addr(buf), BYTES);
}

template <int NY, int H>
constexpr size_t rplane_fft_smem() {
  return ((size_t)RPlane<NY, H>::BUF + NY + H + (H + 1)) * sizeof(cf) + sizeof(unsigned long long);
}

// First-stage source of the forward x transform of the y and z terms: the
// sum of the two fields' pencils (each already times its divergence factor)
struct GPencilsSum {
  const cf *a, *b;
  long base, estride;
  int nvalid;
  __device__ __forceinline__ cf load(int w, int e) const {
    if (w >= nvalid) return cf{0.f, 0.f};
    const long q = base + w + e * estride;
    const cf u = a[q], v = b[q];
    return cf{u.x + v.x, u.y + v.y};
  }
};
// Last-stage sink of that transform: acc += X
struct AccAdd {
  cf *acc;
  int sw, nvalid;
  __device__ __forceinline__ void store(int w, int e, cf v) const {
    if (w >= nvalid) return;
    cf a = acc[e * sw + w];
    a.x += v.x;
    a.y += v.y;
    acc[e * sw + w] = a;
  }
};

// Last-stage sink of the forward x transforms: acc += k_D exp(-i dx k_D/2) X_D
template <int D>
struct DivAcc {
  cf *acc;
  const int *pj, *pkz;
  int sw, nvalid;
  Grid g;
  __device__ __forceinline__ void store(int w, int e, cf v) const {
    if (w >= nvalid) return;
    const int j = pj[w], kz = pkz[w];
    const float kd = g.wavef[D] * (float)((D == 0) ? kx_of(g, e) : (D == 1) ? ky_of(g, j) : kz);
    float cs, sn;
    shift_of(g, D, (D == 0) ? e : (D == 1) ? j : kz, cs, sn);
    const float ksr = kd * cs, ksi = -kd * sn;
    cf a = (D == 0) ? cf{0.f, 0.f} : acc[e * sw + w];
    a.x += v.x * ksr - v.y * ksi;
    a.y += v.x * ksi + v.y * ksr;
    acc[e * sw + w] = a;
  }
};

template <int N, int KWT, bool THREE>
__global__ void __launch_bounds__(512) k_kop_xfwd(Grid g, const float *w0, const float *wa, const float *wb,
                                                  float *out, int mode, const float *other, double *partials,
                                                  double *finals, unsigned *counter, const cf *__restrict__ twx,
                                                  const double *ks) {
  extern __shared__ unsigned char smem_raw[];
  const int sw = KWT + 1;
  cf *tws = reinterpret_cast<cf *>(smem_raw);
  cf *acc = tws + N;
  cf *ta = acc + N * sw;
  cf *tb = ta + N * sw;
  const int nq = g.ny * g.hnz;
  const int q0 = blockIdx.x * KWT;
  const int nvalid = nq - q0 < KWT ? nq - q0 : KWT;
  const int lin = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  __shared__ int pj[KWT], pkz[KWT];
  load_table(tws, twx, N);
  pencil_coords<KWT>(g, q0, pj, pkz);
  __syncthreads();
  // KOP_CG: the dot is weighted by the preconditioner m(k) (1/eps_ref from ks)
  const float ieps = (mode == KOP_CG) ? (float)__ldcg(ks + KS_IEPS) : 0.f;
  float s0 = 0.f, s1 = 0.f;  // the thread's few terms in FP32; blocks and their sum in FP64
  static_assert(N / 8 <= 512 / KWT, "xblock(N) = KWT x N/8 threads");
  constexpr int XPT = 8;
  cf lo[XPT];  // the dot operands: loaded first, in flight during the transforms
#pragma unroll
  for (int u = 0; u < XPT; u++) {
    const int it = lin + u * nthr;
    const int w = it % KWT, e = it / KWT;
    lo[u] = cf{0.f, 0.f};
    if (mode == KOP_NONE || w >= nvalid) continue;
    lo[u] = ldw(other, (long)e * nq + q0 + w, read_weight(g, e, pj[w], pkz[w]));
  }
  // the x term (w0, times its divergence factor here), then the y and z
  // terms (wa + wb, their factors taken by the plane pass) in one transform;
  // with THREE (the split plane step) the y and z terms each transformed and
  // times their divergence factors here
  block_fft<float, N, KWT>(GPencils<float>{reinterpret_cast<cf *>(const_cast<float *>(w0)), (long)q0, 1, (long)nq, nvalid},
                          DivAcc<0>{acc, pj, pkz, sw, nvalid, g}, ta, tb, sw, tws, false);
  if constexpr (THREE) {
    block_fft<float, N, KWT>(GPencils<float>{reinterpret_cast<cf *>(const_cast<float *>(wa)), (long)q0, 1, (long)nq, nvalid},
                            DivAcc<1>{acc, pj, pkz, sw, nvalid, g}, ta, tb, sw, tws, false);
    block_fft<float, N, KWT>(GPencils<float>{reinterpret_cast<cf *>(const_cast<float *>(wb)), (long)q0, 1, (long)nq, nvalid},
                            DivAcc<2>{acc, pj, pkz, sw, nvalid, g}, ta, tb, sw, tws, false);
  } else {
    block_fft<float, N, KWT>(GPencilsSum{reinterpret_cast<const cf *>(wa), reinterpret_cast<const cf *>(wb), (long)q0,
                                         (long)nq, nvalid},
                            AccAdd{acc, sw, nvalid}, ta, tb, sw, tws, false);
  }
#pragma unroll
  for (int u = 0; u < XPT; u++) {
    const int it = lin + u * nthr;
    const int w = it % KWT, e = it / KWT;
    if (w >= nvalid) continue;
    const int wt = read_weight(g, e, pj[w], pkz[w]);
    if (wt == 0) continue;
    const long idx = (long)e * nq + q0 + w;
    const cf a = acc[e * sw + w];
    const cf val{-a.y, a.x};  // i * acc
    reinterpret_cast<float2 *>(out)[idx] = make_float2(val.x, val.y);
    if (mode == KOP_NONE) continue;
    const float vr = val.x, vi = (wt == 1) ? 0.f : val.y, fw = (float)wt;
    const cf o = lo[u];
    if (mode == KOP_P) {
      s0 += fw * (o.x * vr + o.y * vi);
    } else if (mode == KOP_CG) {
      s0 += fw * precond_m(g, e, pj[w], pkz[w], ieps) * (o.x * vr + o.y * vi);
    } else {
      s0 += fw * (vr * vr + vi * vi);
      s1 += fw * (vr * o.x + vi * o.y);
    }
  }
  if (mode != KOP_NONE) block_partials_final(s0, s1, 1.0 / (double)g.nreal(), partials, finals, counter);
}

// Update kernel: KOP_XR_MPT modes per thread (independent loads), the block's
// modes contiguous in memory; mode t = row*(H+1) + kz with a compile-time row
// length. alpha and omega come from the final sums of the x passes.
constexpr int KOP_XR_TPB = 256, KOP_XR_MPT = 4;
template <int H>
__global__ void __launch_bounds__(KOP_XR_TPB) k_kop_xr(Grid g, float *xt, float *r, const float *p, const float *sv,
                                                     const float *t, const float *r0, double rho,
                                                     const double *fin1, const double *fin2, double *part3,
                                                     double *fin3, unsigned *counter3, double *ks, int maxit) {
  const int lin = threadIdx.x;
  __shared__ float sc[2];  // alpha, omega: two FP64 divisions per block, not per thread
  __shared__ int stop;     // the solve is done: this launch leaves x and r alone
  if (lin == 0) {
    const double r0v = fin1[0], tt = fin2[0], ts = fin2[1];
    const double rk = ks ? __ldcg(ks + KS_RHO) : rho;
    stop = (ks && __ldcg(ks + KS_DONE) != 0.0) ? 1 : 0;
    sc[0] = (float)(rk / r0v);
    sc[1] = (float)((tt > 0.0) ? ts / tt : 0.0);
  }
  __syncthreads();
  if (stop) return;
  if (ks) rho = __ldcg(ks + KS_RHO);  // the last block's update below
  const float alpha = sc[0], w = sc[1];
  constexpr int RL = H + 1;  // modes per z row
  const long nm = g.nmodes();
  const long base = (long)blockIdx.x * (KOP_XR_TPB * KOP_XR_MPT);
  const int lny = __ffs(g.ny) - 1;  // NY is a power of two
  // the thread's few terms are summed in FP32 (FP64 arithmetic is scarce on
  // this GPU); blocks and the final sum over blocks are FP64
  float s0 = 0.f, s1 = 0.f;
#pragma unroll
  for (int k = 0; k < KOP_XR_MPT; k++) {
    const long idx = base + k * KOP_XR_TPB + lin;
    if (idx >= nm) break;
    const int row = (int)(idx / RL), kz = (int)(idx - (long)row * RL);
    const int i = row >> lny, j = row & (g.ny - 1);
    const int wt = read_weight(g, i, j, kz);
    if (wt == 0) continue;
    const cf pp = ldw(p, idx, wt), ss = ldw(sv, idx, wt), tv = ldw(t, idx, wt), xx = ldw(xt, idx, wt);
    const cf a = ldw(r0, idx, wt);
    const cf nx{xx.x + alpha * pp.x + w * ss.x, xx.y + alpha * pp.y + w * ss.y};
    const cf nr{ss.x - w * tv.x, ss.y - w * tv.y};
    reinterpret_cast<float2 *>(xt)[idx] = make_float2(nx.x, nx.y);
    reinterpret_cast<float2 *>(r)[idx] = make_float2(nr.x, nr.y);
    const float fw = (float)wt;
    s0 += fw * (a.x * nr.x + a.y * nr.y);
    s1 += fw * (nr.x * nr.x + nr.y * nr.y);
  }
  const int last = block_partials_final(s0, s1, 1.0 / (double)g.nreal(), part3, fin3, counter3);
  if (last && ks) {
    __syncthreads();
    if (lin == 0) {
      // the next iteration's scalars, as the host loop would form them, and
      // the stop test (converged, non-finite, iteration limit, or a restart
      // that the host must perform)
      const double r0v = __ldcg(fin1), tt = __ldcg(fin2), ts = __ldcg(fin2 + 1);
      const double alpha = rho / r0v, w = (tt > 0.0) ? ts / tt : 0.0;
      const double rho_new = __ldcg(fin3), rr = __ldcg(fin3 + 1);
      const double it = ks[KS_ITERS] + 1.0;
      ks[KS_BETA] = (rho_new / rho) * (alpha / w);
      ks[KS_OMEGA] = w;
      ks[KS_RHO] = rho_new;
      ks[KS_ITERS] = it;
      ks[KS_RR] = rr;
      double done = 0.0;
      if (!(rr > ks[KS_TOL2]) || !isfinite(rr) || it >= (double)maxit) done = 1.0;
      else if (fabs(rho_new) < ks[KS_RESTART]) done = 2.0;
      ks[KS_DONE] = done;
    }
  }
}

// Update kernel of the preconditioned CG (the inner solve's alternative to
// BiCGSTAB: the operator is symmetric, A = -(D+)^* eps D+, and so is the
// spectral preconditioner m(k)). In the x~ form p = M^-1 p~, x = M^-1 x~:
// alpha = rho / (M^-1 p~, q) with q = B p~ (fin_pq, from k_kop_xfwd's KOP_CG
// dot); x~ += alpha p~; r -= alpha q; then rho' = (r, M^-1 r) and |r|^2,
// and the last block forms beta = rho'/rho (k_kop_xinv's KOP_PC update makes
// p~ = r + beta p~) and the stop test. init: no update, only
// rho and |r|^2 of the starting residual (beta = 0: p~ = r).
template <int H>
__global__ void __launch_bounds__(KOP_XR_TPB) k_kop_cg(Grid g, float *xt, float *r, const float *p, const float *q,
                                                     const double *fin_pq, double *part, double *fin,
                                                     unsigned *counter, double *ks, int maxit, int init,
                                                     cudaGraphConditionalHandle h) {
  const int lin = threadIdx.x;
  __shared__ float sc[2];  // alpha, 1/eps_ref
  __shared__ int stop;     // the solve is done: this launch leaves x and r alone
  if (lin == 0) {
    stop = (__ldcg(ks + KS_DONE) != 0.0) ? 1 : 0;
    sc[0] = init ? 0.f : (float)(__ldcg(ks + KS_RHO) / __ldcg(fin_pq));
    sc[1] = (float)__ldcg(ks + KS_IEPS);
  }
  __syncthreads();
  if (stop) {
    // inside the step graph's inner loop: a pass that finds the solve done
    // ends the loop (every pass sets the loop's condition)
    if (h && blockIdx.x == 0 && lin == 0) cudaGraphSetConditional(h, 0u);
    return;
  }
  const float alpha = sc[0], ieps = sc[1];
  constexpr int RL = H + 1;  // modes per z row
  const long nm = g.nmodes();
  const long base = (long)blockIdx.x * (KOP_XR_TPB * KOP_XR_MPT);
  const int lny = __ffs(g.ny) - 1;
  float s0 = 0.f, s1 = 0.f;
#pragma unroll
  for (int k = 0; k < KOP_XR_MPT; k++) {
    const long idx = base + k * KOP_XR_TPB + lin;
    if (idx >= nm) break;
    const int row = (int)(idx / RL), kz = (int)(idx - (long)row * RL);
    const int i = row >> lny, j = row & (g.ny - 1);
    const int wt = read_weight(g, i, j, kz);
    if (wt == 0) continue;
    cf nr = ldw(r, idx, wt);
    if (!init) {
      const cf pp = ldw(p, idx, wt), qq = ldw(q, idx, wt), xx = ldw(xt, idx, wt);
      nr = cf{nr.x - alpha * qq.x, nr.y - alpha * qq.y};
      reinterpret_cast<float2 *>(xt)[idx] = make_float2(xx.x + alpha * pp.x, xx.y + alpha * pp.y);
      reinterpret_cast<float2 *>(r)[idx] = make_float2(nr.x, nr.y);
    }
    const float fw = (float)wt, n2 = nr.x * nr.x + nr.y * nr.y;
    s0 += fw * precond_m(g, i, j, kz, ieps) * n2;
    s1 += fw * n2;
  }
  const int last = block_partials_final(s0, s1, 1.0 / (double)g.nreal(), part, fin, counter);
  if (last) {
    __syncthreads();
    if (lin == 0) {
      const double rho_new = __ldcg(fin), rr = __ldcg(fin + 1);
      const double it = ks[KS_ITERS] + (init ? 0.0 : 1.0);
      ks[KS_BETA] = init ? 0.0 : rho_new / ks[KS_RHO];
      ks[KS_OMEGA] = 0.0;
      ks[KS_RHO] = rho_new;
      ks[KS_ITERS] = it;
      ks[KS_RR] = rr;
      const bool done = !(rr > ks[KS_TOL2]) || !isfinite(rr) || !isfinite(rho_new) || it >= (double)maxit;
      ks[KS_DONE] = done ? 1.0 : 0.0;
      // the step graph's inner loop continues while the solve is not done
      // (at most maxit passes: KS_ITERS counts them)
      if (h) cudaGraphSetConditional(h, done ? 0u : 1u);
    }
  }
}

// w_d *= ef_d at the real points (the product of the split plane step)
__global__ void k_kop_eps_mul(Grid g, float *w0, float *w1, float *w2, const float *ef0, const float *ef1,
                              const float *ef2) {
  const long tl = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tl >= g.nreal()) return;
  int i, j, k;
  real_ijk(g, (unsigned)tl, i, j, k);
  const long im = gidx(g, i, j, k);
  w0[im] *= ef0[im];
  w1[im] *= ef1[im];
  w2[im] *= ef2[im];
}

__global__ void k_kop_eps_faces(Grid g, const float *eps, float *ef0, float *ef1, float *ef2, float half) {
  const long tl = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tl >= g.nreal()) return;
  int i, j, k;
  real_ijk(g, (unsigned)tl, i, j, k);
  const long im = gidx(g, i, j, k);
  const float e0 = eps[im];
  ef0[im] = half * (eps[gidx(g, (i + 1) % g.nx, j, k)] + e0);
  ef1[im] = half * (eps[gidx(g, i, (j + 1) % g.ny, k)] + e0);
  ef2[im] = half * (eps[gidx(g, i, j, (k + 1) % g.nz)] + e0);
}

size_t xpass_smem(int n, int kw) { return ((size_t)n + 3 * (size_t)n * (kw + 1)) * sizeof(cf); }
size_t plane_smem_f(int ny, int h) { return kplane_smem(ny, h); }
constexpr size_t KOP_PLANE_SMEM_MAX = 220 * 1024;

dim3 xblock(int n, int kw) { return dim3(kw, n / 8 < 512 / kw ? n / 8 : 512 / kw); }

template <int N, int KWT, bool THREE>
void set_x_attr() {
  static bool attr = false;  // one attribute call per instantiation
  if (attr) return;
  cudaFuncSetAttribute(k_kop_xinv<N, KWT, THREE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)xpass_smem(N, KWT));
  cudaFuncSetAttribute(k_kop_xfwd<N, KWT, THREE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)xpass_smem(N, KWT));
  attr = true;
}

// pencils per block of the x passes that a mesh edge N offers the tuner
// (N/8 threads per pencil, at most 512 threads per block)
inline bool xkw_ok(int n, int kw) { return (kw == 8 || kw == 16 || kw == 32) && n / 8 * kw <= 512 && (n == 64 || n == 128 || kw == 16); }

template <int N, int KWT, bool THREE = false>
void launch_xinv(const Grid &g, int mode, float *vec, const float *r, const float *v, double beta, double omega,
                 double rho, const double *fin, float ieps, float *w0, float *w1, float *w2, float *w3,
                 const cf *twx, const double *ks, cudaStream_t s) {
  set_x_attr<N, KWT, THREE>();
  k_kop_xinv<N, KWT, THREE><<<div_up((long)g.ny * g.hnz, KWT), xblock(N, KWT), xpass_smem(N, KWT), s>>>(
      g, mode, vec, r, v, (float)beta, (float)omega, rho, fin, ieps, w0, w1, w2, w3, twx, ks);
}
template <int N, int KWT, bool THREE = false>
void launch_xfwd(const Grid &g, const float *w0, const float *wa, const float *wb, float *out, int mode,
                 const float *other, double *partials, double *finals, unsigned *counter, const cf *twx,
                 const double *ks, cudaStream_t s) {
  set_x_attr<N, KWT, THREE>();
  k_kop_xfwd<N, KWT, THREE><<<div_up((long)g.ny * g.hnz, KWT), xblock(N, KWT), xpass_smem(N, KWT), s>>>(
      g, w0, wa, wb, out, mode, other, partials, finals, counter, twx, ks);
}

// the register plane pass covers NY in {64, 128} and NZ/2 in {32, 64}
template <int NY, int H>
constexpr bool rplane_ok() {
  return (NY == 64 || NY == 128) && (H == 32 || H == 64) && H <= NY;
}

template <int NY, int H>
void launch_plane_nh(const FFTPlan<float> &p, float *w0, float *w1, float *w2, float *w3, const float *ef0,
                     const float *ef1, const float *ef2, int *err, cudaStream_t s, int test_wait = 0,
                     bool smem_kernel = false) {
  if constexpr (rplane_ok<NY, H>()) {
    if (!smem_kernel) {
      constexpr size_t sm = rplane_smem<NY, H>();
      static bool attr = false;  // one attribute call per instantiation
      if (!attr) {
        cudaFuncSetAttribute(k_kop_plane_r<NY, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        attr = true;
      }
      count_launch(fld<float>(p.g, 8));
      probe_begin(PROBE_KOP_PLANE, s);
      k_kop_plane_r<NY, H><<<dim3(p.g.nx, 3), RPlane<NY, H>::NT, sm, s>>>(
          p.g, w0, w1, w2, w3, ef0, ef1, ef2, p.tw_y, p.tw_z, p.tw_post, err, test_wait);
      // algorithmic bytes: the half spectra of the x gradient and of M in,
      // eps_face_d in and the three components' half spectra out
      probe_end(PROBE_KOP_PLANE, 8.0 * sizeof(float) * (double)p.g.nreal(), s);
      return;
    }
  }
  {
    const size_t sm = plane_smem_f(NY, H);
    static bool attr = false;  // one attribute call per instantiation
    if (!attr) {
      cudaFuncSetAttribute(k_kop_plane<NY, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      attr = true;
    }
    count_launch(fld<float>(p.g, 8));
    probe_begin(PROBE_KOP_PLANE, s);
    k_kop_plane<NY, H><<<dim3(p.g.nx, 3), 1024, sm, s>>>(p.g, w0, w1, w2, w3, ef0, ef1, ef2, p.tw_y, p.tw_z,
                                                               p.tw_post, err);
    probe_end(PROBE_KOP_PLANE, 8.0 * sizeof(float) * (double)p.g.nreal(), s);
  }
}

template <int NY>
void launch_plane_n(const FFTPlan<float> &p, float *w0, float *w1, float *w2, float *w3, const float *ef0,
                    const float *ef1, const float *ef2, int *err, cudaStream_t s, bool smem_kernel) {
  switch (p.g.nz / 2) {
    case 8: launch_plane_nh<NY, 8>(p, w0, w1, w2, w3, ef0, ef1, ef2, err, s, 0, smem_kernel); break;
    case 16: launch_plane_nh<NY, 16>(p, w0, w1, w2, w3, ef0, ef1, ef2, err, s, 0, smem_kernel); break;
    case 32: launch_plane_nh<NY, 32>(p, w0, w1, w2, w3, ef0, ef1, ef2, err, s, 0, smem_kernel); break;
    default: launch_plane_nh<NY, 64>(p, w0, w1, w2, w3, ef0, ef1, ef2, err, s, 0, smem_kernel); break;
  }
}

}  // namespace

template <int NY, int H>
bool launch_rplane_fft(const FFTPlan<float> &p, const FieldBatch<float> &fb, bool inverse, int *err, cudaStream_t s) {
  if constexpr (!rplane_ok<NY, H>()) {
    return false;
  } else {
    constexpr size_t sm = rplane_fft_smem<NY, H>();
    static bool attr = false;  // one attribute call per instantiation
    if (!attr) {
      cudaFuncSetAttribute(k_plane_c2r_r<NY, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      cudaFuncSetAttribute(k_plane_r2c_r<NY, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      attr = true;
    }
    count_launch(fld<float>(p.g, 1.0 * fb.n));
    if (inverse) {
      const float scale = (float)(1.0 / ((double)p.g.nx * p.g.ny * p.g.nz));
      k_plane_c2r_r<NY, H><<<dim3(p.g.nx, fb.n), RPlane<NY, H>::NT, sm, s>>>(fb, p.tw_y, p.tw_z, p.tw_post, scale,
                                                                            err);
    } else {
      k_plane_r2c_r<NY, H><<<dim3(p.g.nx, fb.n), RPlane<NY, H>::NT, sm, s>>>(fb, p.tw_y, p.tw_z, p.tw_post, err);
    }
    return true;
  }
}

bool fft_plane_r(const FFTPlan<float> &p, const FieldBatch<float> &fb, bool inverse, cudaStream_t s) {
  if (!p.err || fb.n < 1) return false;
  const int ny = p.g.ny, h = p.g.nz / 2;
  if (ny == 128 && h == 64) return launch_rplane_fft<128, 64>(p, fb, inverse, p.err, s);
  if (ny == 128 && h == 32) return launch_rplane_fft<128, 32>(p, fb, inverse, p.err, s);
  if (ny == 64 && h == 64) return launch_rplane_fft<64, 64>(p, fb, inverse, p.err, s);
  if (ny == 64 && h == 32) return launch_rplane_fft<64, 32>(p, fb, inverse, p.err, s);
  return false;
}

// an x-plane of one component fits in one block's shared memory
bool kop_plane_fits(const Grid &g) {
  return g.ny <= 128 && g.nz <= 128 && plane_smem_f(g.ny, g.nz / 2) <= KOP_PLANE_SMEM_MAX;
}
bool kop_supported(const Grid &g) {
  // larger planes (up to 256^2) take the split plane step: the plain
  // transform's separate y-pencil and z-row passes around the product
  return kop_plane_fits(g) || (g.nx <= 256 && g.ny <= 256 && g.nz <= 256);
}

// (an upper bound over the x-pass variants: at least 8 pencils per block)
int kop_pencil_blocks(const Grid &g) { return (int)div_up((long)g.ny * g.hnz, 8); }

void kop_eps_faces(const Grid &g, const float *eps, float *ef0, float *ef1, float *ef2, cudaStream_t s) {
  // 0.5, times the inverse transform's 1/N where the plane kernels apply the
  // product (N a power of two: both products are exact, so the result is
  // the one of scaling the transformed row first); the split plane step's
  // transforms scale themselves
  const double sc = kop_plane_fits(g) ? 1.0 / ((double)g.nx * g.ny * g.nz) : 1.0;
  count_launch(fld<float>(g, 4));
  k_kop_eps_faces<<<div_up(g.nreal(), 256), 256, 0, s>>>(g, eps, ef0, ef1, ef2, (float)(0.5 * sc));
}

void kop_xinv(const FFTPlan<float> &p, int mode, float *vec, const float *r, const float *v, double beta,
              double omega, double rho, const double *fin, double eps_ref, float *w0, float *w1, float *w2,
              float *w3, cudaStream_t s, const double *ks, const KopTiles &t) {
  const Grid &g = p.g;
  const float ieps = (float)(1.0 / eps_ref);
  const int kw = xkw_ok(g.nx, t.xinv_kw) ? t.xinv_kw : 16;
  // the split plane step takes the three gradients (no factors in its passes)
  const int three = kop_plane_fits(g) ? 0 : 1;
  const double nfld = (mode == KOP_P ? 6.0 : (mode == KOP_S || mode == KOP_PC) ? 5.0 : 3.0) + three;
  count_launch(fld<float>(g, nfld));
  probe_begin(PROBE_KOP_XINV, s);
#define KOP_XINV(N, W) launch_xinv<N, W>(g, mode, vec, r, v, beta, omega, rho, fin, ieps, w0, w1, w2, w3, p.tw_x, ks, s)
#define KOP_XINV3(N) \
  launch_xinv<N, 16, true>(g, mode, vec, r, v, beta, omega, rho, fin, ieps, w0, w1, w2, w3, p.tw_x, ks, s)
  if (three) {  // the split plane step: 16 pencils per block
    switch (g.nx) {
      case 16: KOP_XINV3(16); break;
      case 32: KOP_XINV3(32); break;
      case 64: KOP_XINV3(64); break;
      case 128: KOP_XINV3(128); break;
      case 256: KOP_XINV3(256); break;
    }
  } else switch (g.nx) {
    case 16: KOP_XINV(16, 16); break;
    case 32: KOP_XINV(32, 16); break;
    case 64:
      if (kw == 8) KOP_XINV(64, 8);
      else if (kw == 32) KOP_XINV(64, 32);
      else KOP_XINV(64, 16);
      break;
    case 128:
      if (kw == 8) KOP_XINV(128, 8);
      else if (kw == 32) KOP_XINV(128, 32);
      else KOP_XINV(128, 16);
      break;
    case 256: KOP_XINV(256, 16); break;
  }
#undef KOP_XINV
#undef KOP_XINV3
  // algorithmic bytes: r, v (and p) in, the updated vector and 2 fields out
  // (3 for the split plane step; KOP_PC: r and p~ in)
  probe_end(PROBE_KOP_XINV, nfld * sizeof(float) * (double)g.nreal(), s);
}

void kop_plane(const FFTPlan<float> &p, float *w0, float *w1, float *w2, float *w3, const float *ef0,
               const float *ef1, const float *ef2, int *err, cudaStream_t s, const KopTiles &t) {
  if (!kop_plane_fits(p.g)) {
    // the split plane step on the three gradients (w0, w2, w3 from
    // kop_xinv): inverse y and z transforms (scaled), the face permittivity
    // product in real space, forward z and y transforms (the divergence
    // factors are kop_xfwd's)
    FieldBatch<float> fb{};
    fb.p[0] = w0;
    fb.p[1] = w2;
    fb.p[2] = w3;
    fb.n = 3;
    fft_pass(p, fb, 3, s);
    count_launch(fld<float>(p.g, 9));
    k_kop_eps_mul<<<(unsigned)div_up(p.g.nreal(), 256), 256, 0, s>>>(p.g, w0, w2, w3, ef0, ef1, ef2);
    fft_pass(p, fb, 0, s);
    return;
  }
  const bool smem = t.plane_smem != 0;
  switch (p.g.ny) {
    case 16: launch_plane_n<16>(p, w0, w1, w2, w3, ef0, ef1, ef2, err, s, smem); break;
    case 32: launch_plane_n<32>(p, w0, w1, w2, w3, ef0, ef1, ef2, err, s, smem); break;
    case 64: launch_plane_n<64>(p, w0, w1, w2, w3, ef0, ef1, ef2, err, s, smem); break;
    default: launch_plane_n<128>(p, w0, w1, w2, w3, ef0, ef1, ef2, err, s, smem); break;
  }
}

KopTiles kop_autotune(const FFTPlan<float> &p, float *vec, float *w0, float *w1, float *w2, float *w3,
                      const float *ef0, const float *ef1, const float *ef2, float *out, int *err, cudaStream_t s,
                      double *us) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int>, std::pair<KopTiles, std::vector<double>>> cache;
  const Grid &g = p.g;
  const auto key = std::make_tuple(g.nx, g.ny, g.nz);
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
      if (us)
        for (int k = 0; k < 8; k++) us[k] = it->second.second[k];
      return it->second.first;
    }
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto time_us = [&](auto launch) -> double {
    launch();
    cudaEventRecord(e0, s);
    for (int r = 0; r < 5; r++) launch();
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    return 1000.0 * ms / 5.0;
  };
  std::vector<double> t(8, 0.0);
  const int kws[3] = {8, 16, 32};
  KopTiles best;  // the defaults (16 pencils) unless a candidate is clearly faster
  for (int c = 0; c < 3; c++) {
    KopTiles v;
    v.xinv_kw = v.xfwd_kw = kws[c];
    if (!xkw_ok(g.nx, kws[c])) continue;
    t[c] = time_us([&]() {
      kop_xinv(p, KOP_NONE, vec, nullptr, nullptr, 0, 0, 0, nullptr, 1.0, w0, w1, w2, w3, s, nullptr, v);
    });
    t[3 + c] = time_us([&]() { kop_xfwd(p, w0, w2, w3, out, KOP_NONE, nullptr, nullptr, nullptr, nullptr, s, v); });
  }
  // a candidate replaces the default when it is more than 3% faster in this
  // isolated timing (near-ties went either way between runs, and inside the
  // step the default was the faster of two tied shapes)
  auto pick = [&](const double *tt) {
    int b = 1;
    for (int c = 0; c < 3; c++)
      if (tt[c] > 0.0 && tt[c] < 0.97 * tt[1] && tt[c] < tt[b]) b = c;
    return kws[b];
  };
  best.xinv_kw = pick(&t[0]);
  best.xfwd_kw = pick(&t[3]);
  KopTiles reg, sh;
  sh.plane_smem = 1;
  const bool has_reg = (g.ny == 64 || g.ny == 128) && (g.nz / 2 == 32 || g.nz / 2 == 64) && g.nz / 2 <= g.ny;
  if (has_reg) t[6] = time_us([&]() { kop_plane(p, w0, w1, w2, w3, ef0, ef1, ef2, err, s, reg); });
  t[7] = time_us([&]() { kop_plane(p, w0, w1, w2, w3, ef0, ef1, ef2, err, s, sh); });
  best.plane_smem = (has_reg && t[6] <= t[7]) ? 0 : 1;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaMemsetAsync(err, 0, sizeof(int), s);
  {
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = std::make_pair(best, t);
  }
  if (us)
    for (int k = 0; k < 8; k++) us[k] = t[k];
  return best;
}

bool kop_plane_selftest(const FFTPlan<float> &p, float *w0, float *w1, float *w2, float *w3, const float *ef0,
                        const float *ef1, const float *ef2, int *err, cudaStream_t s) {
  const int ny = p.g.ny, h = p.g.nz / 2;
  if (ny == 128 && h == 64) launch_plane_nh<128, 64>(p, w0, w1, w2, w3, ef0, ef1, ef2, err, s, 1);
  else if (ny == 128 && h == 32) launch_plane_nh<128, 32>(p, w0, w1, w2, w3, ef0, ef1, ef2, err, s, 1);
  else if (ny == 64 && h == 64) launch_plane_nh<64, 64>(p, w0, w1, w2, w3, ef0, ef1, ef2, err, s, 1);
  else if (ny == 64 && h == 32) launch_plane_nh<64, 32>(p, w0, w1, w2, w3, ef0, ef1, ef2, err, s, 1);
  else return false;
  return true;
}

void kop_xfwd(const FFTPlan<float> &p, const float *w0, const float *wa, const float *wb, float *out, int mode,
              const float *other, double *partials, double *finals, unsigned *counter, cudaStream_t s,
              const KopTiles &t, const double *ks) {
  const Grid &g = p.g;
  const int kw = xkw_ok(g.nx, t.xfwd_kw) ? t.xfwd_kw : 16;
  count_launch(fld<float>(g, mode == KOP_NONE ? 4.0 : 5.0));
  probe_begin(PROBE_KOP_XFWD, s);
  const int three = kop_plane_fits(g) ? 0 : 1;
#define KOP_XFWD(N, W) launch_xfwd<N, W>(g, w0, wa, wb, out, mode, other, partials, finals, counter, p.tw_x, ks, s)
#define KOP_XFWD3(N) \
  launch_xfwd<N, 16, true>(g, w0, wa, wb, out, mode, other, partials, finals, counter, p.tw_x, ks, s)
  if (three) {  // the split plane step: 16 pencils per block
    switch (g.nx) {
      case 16: KOP_XFWD3(16); break;
      case 32: KOP_XFWD3(32); break;
      case 64: KOP_XFWD3(64); break;
      case 128: KOP_XFWD3(128); break;
      case 256: KOP_XFWD3(256); break;
    }
  } else switch (g.nx) {
    case 16: KOP_XFWD(16, 16); break;
    case 32: KOP_XFWD(32, 16); break;
    case 64:
      if (kw == 8) KOP_XFWD(64, 8);
      else if (kw == 32) KOP_XFWD(64, 32);
      else KOP_XFWD(64, 16);
      break;
    case 128:
      if (kw == 8) KOP_XFWD(128, 8);
      else if (kw == 32) KOP_XFWD(128, 32);
      else KOP_XFWD(128, 16);
      break;
    case 256: KOP_XFWD(256, 16); break;
  }
#undef KOP_XFWD
#undef KOP_XFWD3
  // algorithmic bytes: the 3 terms' fields and the dot operand in, the output vector out
  probe_end(PROBE_KOP_XFWD, (mode == KOP_NONE ? 4.0 : 5.0) * sizeof(float) * (double)g.nreal(), s);
}

int kop_xr_blocks(const Grid &g) { return (int)div_up(g.nmodes(), KOP_XR_TPB * KOP_XR_MPT); }

void kop_xr(const Grid &g, float *xt, float *r, const float *p, const float *sv, const float *t, const float *r0,
            double rho, const double *fin1, const double *fin2, double *part3, double *fin3, unsigned *counter3,
            cudaStream_t s, double *ks, int maxit) {
  const unsigned nb = (unsigned)kop_xr_blocks(g);
  count_launch(fld<float>(g, 7));
#define KOP_XR(HH)                                                                                            \
  case HH:                                                                                                    \
    k_kop_xr<HH><<<nb, KOP_XR_TPB, 0, s>>>(g, xt, r, p, sv, t, r0, rho, fin1, fin2, part3, fin3, counter3, ks, \
                                           maxit);                                                              \
    break;
  switch (g.nz / 2) {
    KOP_XR(8)
    KOP_XR(16)
    KOP_XR(32)
    KOP_XR(64)
    KOP_XR(128)
  }
#undef KOP_XR
}

void kop_cg(const Grid &g, float *xt, float *r, const float *p, const float *q, const double *fin_pq, double *part,
            double *fin, unsigned *counter, cudaStream_t s, double *ks, int maxit, bool init,
            cudaGraphConditionalHandle h) {
  const unsigned nb = (unsigned)kop_xr_blocks(g);
  count_launch(fld<float>(g, init ? 1.0 : 6.0));
#define KOP_CG(HH)                                                                                             \
  case HH:                                                                                                     \
    k_kop_cg<HH><<<nb, KOP_XR_TPB, 0, s>>>(g, xt, r, p, q, fin_pq, part, fin, counter, ks, maxit, init ? 1 : 0, h); \
    break;
  switch (g.nz / 2) {
    KOP_CG(8)
    KOP_CG(16)
    KOP_CG(32)
    KOP_CG(64)
    KOP_CG(128)
  }
#undef KOP_CG
}

}  // namespace icep
