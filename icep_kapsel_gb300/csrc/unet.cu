// unet.cu -- see unet.cuh.
//
// Voxel v of an n^3 grid (n = 2^lg) is v = (x << 2lg) | (y << lg) | z;
// activations are [v][c]. Tap t = 9(dx+1) + 3(dy+1) + (dz+1) reads the
// neighbour (x+dx, y+dy, z+dz) (periodic); FP32 weights are W[t][ci][co].
#include <stdint.h>

#include <cmath>
#include <random>
#include <vector>

#include "unet.cuh"

namespace icep {

namespace {

constexpr int CONV_WARPS = 4;  // warps per block of the tensor-core convolution
constexpr int WG_CH = 128;     // voxels per block of the weight-gradient reduction

__device__ __forceinline__ int vox(int lg, int x, int y, int z) { return (x << (2 * lg)) | (y << lg) | z; }
__device__ __forceinline__ void vcoord(int lg, int v, int &x, int &y, int &z) {
  const int m = (1 << lg) - 1;
  z = v & m;
  y = (v >> lg) & m;
  x = v >> (2 * lg);
}
__device__ __forceinline__ void tap(int t, int &dx, int &dy, int &dz) {
  dx = t / 9 - 1;
  dy = (t / 3) % 3 - 1;
  dz = t % 3 - 1;
}
__device__ __forceinline__ uint32_t ld32(const bf16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

__device__ __forceinline__ void mma_bf16(float *d, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// ---- tensor-core convolution ---------------------------------------------
// out[v][co] = act(bias[co] + sum_t sum_ci in[v + s_t][ci] Wk[t][co][ci]),
// in = cat(a (CINA channels, this grid), up(b) (CINB channels, the grid of
// half the edge, nearest up-sampling)). One warp computes 16 voxels x COUT
// with m16n8k16 BF16 MMAs (FP32 accumulators).
template <int CINA, int CINB, int COUT, bool OUT_F32, bool RELU>
__global__ void __launch_bounds__(CONV_WARPS * 32) k_conv_mma(int lg, const bf16 *__restrict__ a,
                                                             const bf16 *__restrict__ b, const bf16 *__restrict__ W,
                                                             const float *__restrict__ bias, void *out) {
  constexpr int CIN = CINA + CINB;
  constexpr int KC = CIN / 16;
  constexpr int NT = COUT / 8;
  static_assert(CINA % 16 == 0 && CINB % 16 == 0 && COUT % 8 == 0, "channel counts");
  const int V = 1 << (3 * lg);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = lane >> 2, tig = lane & 3;
  const int v0 = (blockIdx.x * CONV_WARPS + warp) * 16;
  if (v0 >= V) return;
  const int va = v0 + gid, vb = va + 8;
  int xa, ya, za, xb, yb, zb;
  vcoord(lg, va, xa, ya, za);
  vcoord(lg, vb, xb, yb, zb);
  const int m = (1 << lg) - 1;
  float acc[NT][4];
#pragma unroll
  for (int j = 0; j < NT; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll 1
  for (int t = 0; t < 27; t++) {
    int dx, dy, dz;
    tap(t, dx, dy, dz);
    const int ax = (xa + dx) & m, ay = (ya + dy) & m, az = (za + dz) & m;
    const int bx = (xb + dx) & m, by = (yb + dy) & m, bz = (zb + dz) & m;
    const int na = vox(lg, ax, ay, az), nb = vox(lg, bx, by, bz);
    const bf16 *wt = W + (long)t * COUT * CIN + tig * 2;
#pragma unroll
    for (int kc = 0; kc < KC; kc++) {
      uint32_t a0, a1, a2, a3;
      if (kc * 16 < CINA) {
        const int c = kc * 16 + tig * 2;
        a0 = ld32(a + (long)na * CINA + c);
        a1 = ld32(a + (long)nb * CINA + c);
        a2 = ld32(a + (long)na * CINA + c + 8);
        a3 = ld32(a + (long)nb * CINA + c + 8);
      } else {
        const int c = kc * 16 - CINA + tig * 2;
        const int ha = vox(lg - 1, ax >> 1, ay >> 1, az >> 1), hb = vox(lg - 1, bx >> 1, by >> 1, bz >> 1);
        a0 = ld32(b + (long)ha * CINB + c);
        a1 = ld32(b + (long)hb * CINB + c);
        a2 = ld32(b + (long)ha * CINB + c + 8);
        a3 = ld32(b + (long)hb * CINB + c + 8);
      }
#pragma unroll
      for (int j = 0; j < NT; j++) {
        const bf16 *wp = wt + (long)(j * 8 + gid) * CIN + kc * 16;
        mma_bf16(acc[j], a0, a1, a2, a3, ld32(wp), ld32(wp + 8));
      }
    }
  }
#pragma unroll
  for (int j = 0; j < NT; j++) {
    const int co = j * 8 + tig * 2;
    const float b0 = bias ? bias[co] : 0.f, b1 = bias ? bias[co + 1] : 0.f;
    float d0 = acc[j][0] + b0, d1 = acc[j][1] + b1, d2 = acc[j][2] + b0, d3 = acc[j][3] + b1;
    if (RELU) {
      d0 = fmaxf(d0, 0.f);
      d1 = fmaxf(d1, 0.f);
      d2 = fmaxf(d2, 0.f);
      d3 = fmaxf(d3, 0.f);
    }
    if (OUT_F32) {
      float *o = static_cast<float *>(out);
      *reinterpret_cast<float2 *>(o + (long)va * COUT + co) = make_float2(d0, d1);
      *reinterpret_cast<float2 *>(o + (long)vb * COUT + co) = make_float2(d2, d3);
    } else {
      bf16 *o = static_cast<bf16 *>(out);
      *reinterpret_cast<__nv_bfloat162 *>(o + (long)va * COUT + co) = __floats2bfloat162_rn(d0, d1);
      *reinterpret_cast<__nv_bfloat162 *>(o + (long)vb * COUT + co) = __floats2bfloat162_rn(d2, d3);
    }
  }
}

// ---- tcgen05 convolution (forward) ------------------------------------------
// out[v][co] = act(bias[co] + sum_t sum_ci in[v + s_t][ci] Wk[t][co][ci]) as an
// implicit GEMM on the 5th-generation tensor cores: a CTA owns 128 voxels
// (M = 128), N = COUT, and walks the 27 taps; per tap the 128 x CIN operand
// rows (the tap's neighbours, cat/up-sampled sources as in k_conv_mma) and
// the COUT x CIN weights are staged in shared memory in the K-major
// no-swizzle core-matrix layout (8 rows x 16 bytes per core matrix), and one
// thread issues CIN/16 tcgen05.mma (kind::f16, BF16 x BF16 -> FP32) into a
// TMEM accumulator. Operand buffers are double-buffered; a tcgen05.commit per
// tap arrives on that buffer's mbarrier, which the threads wait on (bounded)
// before refilling it. The epilogue reads the accumulator with tcgen05.ld.
constexpr int TC_M = 128;
__device__ __forceinline__ uint32_t sh_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
// byte offset of element (row, k) of a K-major no-swizzle tile with KG k-groups
__device__ __forceinline__ int tc_off(int row, int k, int KG) {
  return (((row >> 3) * KG + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1);
}
// shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets between core matrices, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}
// instruction descriptor of kind::f16: FP32 accumulate, BF16 A and B, both K-major
template <int M, int N>
__host__ __device__ constexpr uint32_t tc_idesc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ unsigned long long tc_clock() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Wait for phase `parity` of the mbarrier for at most `limit_ns` of
// %globaltimer time; false on timeout.
__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity, unsigned long long limit_ns) {
  const unsigned long long t0 = tc_clock();
  while (true) {
    uint32_t done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done)
                 : "r"(mbar), "r"(parity)
                 : "memory");
    if (done) return true;
    if (tc_clock() - t0 > limit_ns) return false;
  }
}
// MMA-completion limit (a tap's MMAs take microseconds) and the short limit
// of the bounded-wait self-test
constexpr unsigned long long TC_WAIT_NS = 200ull * 1000 * 1000;
constexpr unsigned long long TC_TEST_WAIT_NS = 50ull * 1000;

template <int CINA, int CINB, int COUT, bool RELU>
__global__ void __launch_bounds__(128) k_conv_tc(int lg, const bf16 *__restrict__ a, const bf16 *__restrict__ b,
                                                 const bf16 *__restrict__ W, const float *__restrict__ bias, bf16 *out,
                                                 int *err, int test_wait) {
  constexpr int CIN = CINA + CINB, KG = CIN / 8, KSTEPS = CIN / 16;
  constexpr int NCOL = COUT <= 32 ? 32 : (COUT <= 64 ? 64 : 128);
  constexpr int ABYTES = TC_M * CIN * 2, BBYTES = COUT * CIN * 2;
  static_assert(CINA % 16 == 0 && CINB % 16 == 0 && COUT % 16 == 0 && COUT <= 128, "tcgen05 shapes");
  extern __shared__ __align__(128) unsigned char tsm[];
  // operand buffers: A[buf] at tsm + buf*ABYTES, B[buf] at tsm + 2*ABYTES + buf*BBYTES
  __shared__ __align__(8) unsigned long long mbar[2];
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int V = 1 << (3 * lg), m = (1 << lg) - 1;
  const int v = blockIdx.x * TC_M + tid;  // this thread's voxel row
  const bool valid = v < V;
  int x0 = 0, y0 = 0, z0 = 0;
  if (valid) vcoord(lg, v, x0, y0, z0);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sh_addr(&mbar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sh_addr(&mbar[1])) : "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sh_addr(&tmem_base)),
                 "r"(NCOL)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  // test_wait (the bounded-wait self-test): no MMA is issued, so the first
  // completion wait runs out and the timeout path below must reach the host
  const unsigned long long lim = test_wait ? TC_TEST_WAIT_NS : TC_WAIT_NS;
  bool failed = false;
  for (int t = 0; t < 27; t++) {
    const int buf = t & 1;
    // the MMAs of tap t-2 read this buffer
    const bool late = (t >= 2) && !tc_wait(sh_addr(&mbar[buf]), ((t - 2) >> 1) & 1, lim);
    // operand rows: this thread's voxel neighbour at tap t, CIN channels in 16-byte chunks
    int dx, dy, dz;
    tap(t, dx, dy, dz);
    const int nx = (x0 + dx) & m, ny = (y0 + dy) & m, nz = (z0 + dz) & m;
#pragma unroll
    for (int c = 0; c < KG; c++) {
      uint4 val = make_uint4(0, 0, 0, 0);
      if (valid) {
        if (c * 8 < CINA)
          val = *reinterpret_cast<const uint4 *>(a + (long)vox(lg, nx, ny, nz) * CINA + c * 8);
        else
          val = *reinterpret_cast<const uint4 *>(b + (long)vox(lg - 1, nx >> 1, ny >> 1, nz >> 1) * CINB +
                                                 (c * 8 - CINA));
      }
      *reinterpret_cast<uint4 *>(tsm + buf * ABYTES + tc_off(tid, c * 8, KG)) = val;
    }
    // weights of tap t, Wk[t][co][ci]
    for (int q = tid; q < COUT * KG; q += 128) {
      const int co = q / KG, c = q - co * KG;
      *reinterpret_cast<uint4 *>(tsm + 2 * ABYTES + buf * BBYTES + tc_off(co, c * 8, KG)) =
          *reinterpret_cast<const uint4 *>(W + ((long)t * COUT + co) * CIN + c * 8);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (__syncthreads_or(late)) {
      // a completion did not arrive: report it, let the MMAs of taps t-2
      // and t-1 finish before the accumulator is released, and leave
      if (tid == 0) atomicExch(err, 1);
      tc_wait(sh_addr(&mbar[buf ^ 1]), ((t - 1) >> 1) & 1, lim);
      tc_wait(sh_addr(&mbar[buf]), ((t - 2) >> 1) & 1, lim);
      failed = true;
      break;
    }
    if (tid == 0 && !test_wait) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int kk = 0; kk < KSTEPS; kk++) {
        const uint64_t ad = tc_desc(sh_addr(tsm + buf * ABYTES) + kk * 256, 128, KG * 128);
        const uint64_t bd = tc_desc(sh_addr(tsm + 2 * ABYTES + buf * BBYTES) + kk * 256, 128, KG * 128);
        const uint32_t acc = (t > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                tmem),
            "l"(ad), "l"(bd), "r"(tc_idesc<TC_M, COUT>()), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       sh_addr(&mbar[buf]))
                   : "memory");
    }
  }
  // the last commit (tap 26, buffer 0, its 14th) follows every MMA
  if (!failed && __syncthreads_or(!tc_wait(sh_addr(&mbar[0]), 13 & 1, lim))) {
    if (tid == 0) atomicExch(err, 1);
    tc_wait(sh_addr(&mbar[0]), 13 & 1, lim);
    failed = true;
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // epilogue: warp w holds rows 32w..32w+31 of the accumulator
#pragma unroll
  for (int c0 = 0; c0 < (failed ? 0 : COUT); c0 += 16) {
    uint32_t r[16];
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const int row = warp * 32 + lane;
    const int vr = blockIdx.x * TC_M + row;
    if (vr < V) {
      __nv_bfloat162 o[8];
#pragma unroll
      for (int j = 0; j < 16; j += 2) {
        float d0 = __uint_as_float(r[j]) + bias[c0 + j], d1 = __uint_as_float(r[j + 1]) + bias[c0 + j + 1];
        if (RELU) {
          d0 = fmaxf(d0, 0.f);
          d1 = fmaxf(d1, 0.f);
        }
        o[j / 2] = __floats2bfloat162_rn(d0, d1);
      }
      uint4 *dst = reinterpret_cast<uint4 *>(out + (long)vr * COUT + c0);
      dst[0] = *reinterpret_cast<uint4 *>(&o[0]);
      dst[1] = *reinterpret_cast<uint4 *>(&o[4]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOL) : "memory");
}

// ---- CUDA-core layers ------------------------------------------------------
// first layer: 2 FP32 input channels -> 16 (bias, relu, BF16 out)
__global__ void k_conv_in(int lg, const float *__restrict__ x, const float *__restrict__ W,
                          const float *__restrict__ bias, bf16 *out) {
  __shared__ float sw[27 * 2 * 16], sb[16];
  for (int q = threadIdx.x; q < 27 * 2 * 16; q += blockDim.x) sw[q] = W[q];
  if (threadIdx.x < 16) sb[threadIdx.x] = bias[threadIdx.x];
  __syncthreads();
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= (1 << (3 * lg))) return;
  int x0, y0, z0;
  vcoord(lg, v, x0, y0, z0);
  const int m = (1 << lg) - 1;
  float acc[16];
#pragma unroll
  for (int c = 0; c < 16; c++) acc[c] = sb[c];
  for (int t = 0; t < 27; t++) {
    int dx, dy, dz;
    tap(t, dx, dy, dz);
    const int nb = vox(lg, (x0 + dx) & m, (y0 + dy) & m, (z0 + dz) & m);
    const float2 in = reinterpret_cast<const float2 *>(x)[nb];
#pragma unroll
    for (int c = 0; c < 16; c++) acc[c] += in.x * sw[(t * 2) * 16 + c] + in.y * sw[(t * 2 + 1) * 16 + c];
  }
  __nv_bfloat162 *o = reinterpret_cast<__nv_bfloat162 *>(out + (long)v * 16);
#pragma unroll
  for (int c = 0; c < 16; c += 2) o[c / 2] = __floats2bfloat162_rn(fmaxf(acc[c], 0.f), fmaxf(acc[c + 1], 0.f));
}

// last layer: 16 BF16 channels -> 1 FP32 (bias, no activation)
__global__ void k_conv_out(int lg, const bf16 *__restrict__ in, const float *__restrict__ W,
                           const float *__restrict__ bias, float *y) {
  __shared__ float sw[27 * 16];
  for (int q = threadIdx.x; q < 27 * 16; q += blockDim.x) sw[q] = W[q];
  __syncthreads();
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= (1 << (3 * lg))) return;
  int x0, y0, z0;
  vcoord(lg, v, x0, y0, z0);
  const int m = (1 << lg) - 1;
  float acc = bias[0];
  for (int t = 0; t < 27; t++) {
    int dx, dy, dz;
    tap(t, dx, dy, dz);
    const int nb = vox(lg, (x0 + dx) & m, (y0 + dy) & m, (z0 + dz) & m);
    const __nv_bfloat162 *ip = reinterpret_cast<const __nv_bfloat162 *>(in + (long)nb * 16);
#pragma unroll
    for (int c = 0; c < 16; c += 2) {
      const float2 f = __bfloat1622float2(ip[c / 2]);
      acc += f.x * sw[t * 16 + c] + f.y * sw[t * 16 + c + 1];
    }
  }
  y[v] = acc;
}

// gradient of the last layer's input, masked by relu of that input (d0 > 0):
// gz[v][ci] = [d0[v][ci] > 0] sum_t gy[v - s_t] W[t][ci]
__global__ void k_conv_out_bwd(int lg, const float *__restrict__ gy, const float *__restrict__ W,
                               const bf16 *__restrict__ act, bf16 *gz) {
  __shared__ float sw[27 * 16];
  for (int q = threadIdx.x; q < 27 * 16; q += blockDim.x) sw[q] = W[q];
  __syncthreads();
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= (1 << (3 * lg))) return;
  int x0, y0, z0;
  vcoord(lg, v, x0, y0, z0);
  const int m = (1 << lg) - 1;
  float acc[16];
#pragma unroll
  for (int c = 0; c < 16; c++) acc[c] = 0.f;
  for (int t = 0; t < 27; t++) {
    int dx, dy, dz;
    tap(t, dx, dy, dz);
    const float gv = gy[vox(lg, (x0 - dx) & m, (y0 - dy) & m, (z0 - dz) & m)];
#pragma unroll
    for (int c = 0; c < 16; c++) acc[c] += gv * sw[t * 16 + c];
  }
  const __nv_bfloat162 *ap = reinterpret_cast<const __nv_bfloat162 *>(act + (long)v * 16);
  __nv_bfloat162 *o = reinterpret_cast<__nv_bfloat162 *>(gz + (long)v * 16);
#pragma unroll
  for (int c = 0; c < 16; c += 2) {
    const float2 f = __bfloat1622float2(ap[c / 2]);
    o[c / 2] = __floats2bfloat162_rn(f.x > 0.f ? acc[c] : 0.f, f.y > 0.f ? acc[c + 1] : 0.f);
  }
}

// ---- weight gradients (FP32 on the CUDA cores) ------------------------------
// dW[t][ci][co] += sum_v in[v + s_t][ci] gz[v][co]; db[co] += sum_v gz[v][co].
// Block (chunk of WG_CH voxels, tap t); partial sums go to dW by atomics.
template <typename TA>
__device__ __forceinline__ float tofloat(TA v);
template <>
__device__ __forceinline__ float tofloat<float>(float v) { return v; }
template <>
__device__ __forceinline__ float tofloat<bf16>(bf16 v) { return __bfloat162float(v); }

template <typename TA, typename TZ, int CINA, int CINB, int COUT>
__global__ void __launch_bounds__(256) k_conv_wgrad(int lg, const TA *__restrict__ a, const TA *__restrict__ b,
                                                    const TZ *__restrict__ gz, float *dW, float *db) {
  constexpr int CIN = CINA + CINB;
  extern __shared__ float wsm[];
  float *sa = wsm;              // [WG_CH][CIN]
  float *sz = wsm + WG_CH * CIN;  // [WG_CH][COUT]
  const int t = blockIdx.y;
  const int v0 = blockIdx.x * WG_CH;
  int dx, dy, dz;
  tap(t, dx, dy, dz);
  const int m = (1 << lg) - 1;
  const int nv = min(WG_CH, (1 << (3 * lg)) - v0);  // voxels of this chunk (the last may be short)
  for (int q = threadIdx.x; q < WG_CH * CIN; q += blockDim.x) {
    const int i = q / CIN, c = q - i * CIN;
    if (i >= nv) {
      sa[q] = 0.f;
      continue;
    }
    int x0, y0, z0;
    vcoord(lg, v0 + i, x0, y0, z0);
    const int nx = (x0 + dx) & m, ny = (y0 + dy) & m, nz = (z0 + dz) & m;
    sa[q] = (c < CINA) ? tofloat<TA>(a[(long)vox(lg, nx, ny, nz) * CINA + c])
                       : tofloat<TA>(b[(long)vox(lg - 1, nx >> 1, ny >> 1, nz >> 1) * CINB + (c - CINA)]);
  }
  for (int q = threadIdx.x; q < WG_CH * COUT; q += blockDim.x)
    sz[q] = (q / COUT < nv) ? tofloat<TZ>(gz[(long)v0 * COUT + q]) : 0.f;
  __syncthreads();
  for (int p = threadIdx.x; p < CIN * COUT; p += blockDim.x) {
    const int ci = p / COUT, co = p - ci * COUT;
    float acc = 0.f;
#pragma unroll 8
    for (int i = 0; i < WG_CH; i++) acc += sa[i * CIN + ci] * sz[i * COUT + co];
    atomicAdd(&dW[(long)t * CIN * COUT + p], acc);
  }
  if (t == 0)
    for (int co = threadIdx.x; co < COUT; co += blockDim.x) {
      float acc = 0.f;
      for (int i = 0; i < WG_CH; i++) acc += sz[i * COUT + co];
      atomicAdd(&db[co], acc);
    }
}

// ---- pooling, splits, masks -------------------------------------------------
// out (grid 2^(lg-1)) = mean of the 8 children in `in` (grid 2^lg), C channels
__global__ void k_pool(int lg, int C, const bf16 *__restrict__ in, bf16 *out) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long Vc = 1L << (3 * (lg - 1));
  if (q >= Vc * C) return;
  const int vc = (int)(q / C), c = (int)(q - (long)vc * C);
  int X, Y, Z;
  vcoord(lg - 1, vc, X, Y, Z);
  float s = 0.f;
  for (int k = 0; k < 8; k++)
    s += __bfloat162float(in[(long)vox(lg, 2 * X + (k >> 2), 2 * Y + ((k >> 1) & 1), 2 * Z + (k & 1)) * C + c]);
  out[q] = __float2bfloat16_rn(0.125f * s);
}

// ga[v][c] = tmp[v][c], c < CA (grid 2^lg, tmp has C channels)
__global__ void k_take_cols(long V, int C, int CA, const float *__restrict__ tmp, float *ga) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= V * CA) return;
  const long v = q / CA;
  ga[q] = tmp[v * C + (q - v * CA)];
}

// gb (grid 2^(lg-1), CB channels) = sum over the 8 children of tmp[child][CA + c]
// (the transpose of nearest up-sampling)
__global__ void k_up_adjoint(int lg, int C, int CA, int CB, const float *__restrict__ tmp, float *gb) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long Vc = 1L << (3 * (lg - 1));
  if (q >= Vc * CB) return;
  const int vc = (int)(q / CB), c = (int)(q - (long)vc * CB);
  int X, Y, Z;
  vcoord(lg - 1, vc, X, Y, Z);
  float s = 0.f;
  for (int k = 0; k < 8; k++)
    s += tmp[(long)vox(lg, 2 * X + (k >> 2), 2 * Y + ((k >> 1) & 1), 2 * Z + (k & 1)) * C + CA + c];
  gb[q] = s;
}

// gf[v][c] += gp[parent(v)][c] / 8 (the transpose of average pooling), grid 2^lg
__global__ void k_pool_adjoint_add(int lg, int C, const float *__restrict__ gp, float *gf) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (1L << (3 * lg)) * C) return;
  const int v = (int)(q / C), c = (int)(q - (long)v * C);
  int x0, y0, z0;
  vcoord(lg, v, x0, y0, z0);
  gf[q] += 0.125f * gp[(long)vox(lg - 1, x0 >> 1, y0 >> 1, z0 >> 1) * C + c];
}

// out = act > 0 ? g : 0 (BF16), count values
__global__ void k_relu_mask(long count, const float *__restrict__ g, const bf16 *__restrict__ act, bf16 *out) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= count) return;
  out[q] = __float2bfloat16_rn(__bfloat162float(act[q]) > 0.f ? g[q] : 0.f);
}

// BF16 copies of one layer's weights: wf[t][co][ci] = W[t][ci][co],
// wb[t][ci][co] = W[26 - t][ci][co] (backward-data as a forward convolution)
__global__ void k_pack_layer(int cin, int cout, const float *__restrict__ W, bf16 *wf, bf16 *wb) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= 27 * cin * cout) return;
  const int t = q / (cin * cout), r = q - t * cin * cout;
  const int ci = r / cout, co = r - ci * cout;
  wf[(long)t * cout * cin + co * cin + ci] = __float2bfloat16_rn(W[q]);
  wb[(long)(26 - t) * cin * cout + r] = __float2bfloat16_rn(W[q]);
}

__global__ void k_adam(long n, float *p, const float *g, float *m, float *v, float lr, float b1, float b2, float eps,
                       float bc1, float bc2) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float gq = g[q];
  const float mq = b1 * m[q] + (1.f - b1) * gq;
  const float vq = b2 * v[q] + (1.f - b2) * gq * gq;
  m[q] = mq;
  v[q] = vq;
  p[q] -= lr * (mq / bc1) / (sqrtf(vq / bc2) + eps);
}

// ---- fine <-> coarse --------------------------------------------------------
__global__ void k_unet_input(Grid g, int lgc, const float *__restrict__ eps, const float *__restrict__ r, float ieref,
                             float irms, float *x) {
  const int vc = blockIdx.x * blockDim.x + threadIdx.x;
  if (vc >= (1 << (3 * lgc))) return;
  int X, Y, Z;
  vcoord(lgc, vc, X, Y, Z);
  float se = 0.f, sr = 0.f;
  for (int k = 0; k < 8; k++) {
    const long im = gidx(g, 2 * X + (k >> 2), 2 * Y + ((k >> 1) & 1), 2 * Z + (k & 1));
    se += eps[im];
    sr += r[im];
  }
  reinterpret_cast<float2 *>(x)[vc] = make_float2(0.125f * se * ieref - 1.f, 0.125f * sr * irms);
}

// z[f] += scale * sum of the 8 coarse neighbours with weights (3/4 or 1/4 per axis)
__global__ void k_prolong_add(Grid g, int lgc, const float *__restrict__ y, float scale, float *z) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.nreal()) return;
  const int k = (int)(t & (g.nz - 1)), j = (int)((t / g.nz) & (g.ny - 1)), i = (int)(t / ((long)g.ny * g.nz));
  const int mc = (1 << lgc) - 1;
  const int f[3] = {i, j, k};
  int c0[3], c1[3];
  for (int d = 0; d < 3; d++) {
    c0[d] = f[d] >> 1;
    c1[d] = (f[d] & 1) ? ((c0[d] + 1) & mc) : ((c0[d] - 1) & mc);
  }
  float s = 0.f;
  for (int q = 0; q < 8; q++) {
    const int ax = (q >> 2) ? c1[0] : c0[0], ay = ((q >> 1) & 1) ? c1[1] : c0[1], az = (q & 1) ? c1[2] : c0[2];
    const float w = ((q >> 2) ? 0.25f : 0.75f) * (((q >> 1) & 1) ? 0.25f : 0.75f) * ((q & 1) ? 0.25f : 0.75f);
    s += w * y[vox(lgc, ax, ay, az)];
  }
  z[gidx(g, i, j, k)] += scale * s;
}

// gy[c] = scale * sum over the 4x4x4 fine cells that interpolate from c
__global__ void k_prolong_adjoint(Grid g, int lgc, const float *__restrict__ dz, float scale, float *gy) {
  const int vc = blockIdx.x * blockDim.x + threadIdx.x;
  if (vc >= (1 << (3 * lgc))) return;
  int X, Y, Z;
  vcoord(lgc, vc, X, Y, Z);
  const int C[3] = {X, Y, Z}, N[3] = {g.nx, g.ny, g.nz};
  int fi[3][4];
  for (int d = 0; d < 3; d++)
    for (int o = 0; o < 4; o++) fi[d][o] = (2 * C[d] - 1 + o) & (N[d] - 1);
  const float w[4] = {0.25f, 0.75f, 0.75f, 0.25f};
  float s = 0.f;
  for (int a = 0; a < 4; a++)
    for (int b = 0; b < 4; b++)
      for (int c = 0; c < 4; c++) s += w[a] * w[b] * w[c] * dz[gidx(g, fi[0][a], fi[1][b], fi[2][c])];
  gy[vc] = scale * s;
}

inline unsigned nb256(long n) { return (unsigned)((n + 255) / 256); }

int ilog2(int n) {
  int l = 0;
  while ((1 << l) < n) l++;
  return l;
}

template <int CINA, int CINB, int COUT, bool OUT_F32, bool RELU>
void conv_mma(int lg, const bf16 *a, const bf16 *b, const bf16 *W, const float *bias, void *out, cudaStream_t s) {
  const long V = 1L << (3 * lg);
  count_launch();
  k_conv_mma<CINA, CINB, COUT, OUT_F32, RELU>
      <<<(unsigned)((V / 16 + CONV_WARPS - 1) / CONV_WARPS), CONV_WARPS * 32, 0, s>>>(lg, a, b, W, bias, out);
}

template <int CINA, int CINB, int COUT, bool RELU>
void conv_tc(int lg, const bf16 *a, const bf16 *b, const bf16 *W, const float *bias, bf16 *out, int *err,
             cudaStream_t s, int test_wait = 0) {
  const long V = 1L << (3 * lg);
  constexpr int CIN = CINA + CINB;
  const size_t sm = 2 * (size_t)(TC_M * CIN + COUT * CIN) * sizeof(bf16);
  static bool attr = false;  // one attribute call per instantiation
  if (!attr) {
    cudaFuncSetAttribute(k_conv_tc<CINA, CINB, COUT, RELU>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    attr = true;
  }
  count_launch();
  k_conv_tc<CINA, CINB, COUT, RELU><<<(unsigned)((V + TC_M - 1) / TC_M), 128, sm, s>>>(lg, a, b, W, bias, out, err,
                                                                                    test_wait);
}

template <typename TA, typename TZ, int CINA, int CINB, int COUT>
void conv_wgrad(int lg, const TA *a, const TA *b, const TZ *gz, float *dW, float *db, cudaStream_t s) {
  const long V = 1L << (3 * lg);
  const size_t sm = sizeof(float) * WG_CH * (CINA + CINB + COUT);
  static bool attr = false;  // one attribute call per instantiation
  if (!attr) {
    cudaFuncSetAttribute(k_conv_wgrad<TA, TZ, CINA, CINB, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    attr = true;
  }
  count_launch();
  k_conv_wgrad<TA, TZ, CINA, CINB, COUT>
      <<<dim3((unsigned)((V + WG_CH - 1) / WG_CH), 27), 256, sm, s>>>(lg, a, b, gz, dW, db);
}

}  // namespace

int UNet::init(int n_coarse, unsigned long long seed, cudaStream_t s) {
  n = n_coarse;
  // every level needs at least one 16-voxel tensor-core tile: n/4 >= 4
  if (n < 16 || (n & (n - 1))) return ICEP_ERR_UNSUPPORTED;
  const int ci[L_COUNT] = {2, 16, 16, 32, 32, 64, 96, 48, 16};
  const int co[L_COUNT] = {16, 16, 32, 32, 64, 64, 32, 16, 1};
  long o = 0, ob = 0;
  for (int l = 0; l < L_COUNT; l++) {
    cin[l] = ci[l];
    cout[l] = co[l];
    woff[l] = o;
    boff[l] = o + 27L * ci[l] * co[l];
    o = boff[l] + co[l];
    wbf_off[l] = ob;
    ob += 27L * ci[l] * co[l];
  }
  nparams = o;
  const long V0 = (long)n * n * n, V1 = V0 / 8, V2 = V0 / 64;
  bool ok = true;
  auto fal = [&](float **p, long cnt) { ok = ok && cudaMalloc(p, sizeof(float) * cnt) == cudaSuccess; };
  auto bal = [&](bf16 **p, long cnt) { ok = ok && cudaMalloc(p, sizeof(bf16) * cnt) == cudaSuccess; };
  fal(&params, nparams);
  fal(&grads, nparams);
  fal(&adam_m, nparams);
  fal(&adam_v, nparams);
  bal(&wf, ob);
  bal(&wb, ob);
  fal(&x, 2 * V0);
  fal(&y, V0);
  bal(&e0a, 16 * V0);
  bal(&e0, 16 * V0);
  bal(&p1, 16 * V1);
  bal(&e1a, 32 * V1);
  bal(&e1, 32 * V1);
  bal(&p2, 32 * V2);
  bal(&e2a, 64 * V2);
  bal(&e2, 64 * V2);
  bal(&d1, 32 * V1);
  bal(&d0, 16 * V0);
  fal(&gy, V0);
  fal(&tmp, 48 * V0);
  fal(&g0, 16 * V0);
  fal(&g1, 32 * V1);
  bal(&gz, 16 * V0);
  bal(&gz2, 16 * V0);
  ok = ok && cudaMalloc(&err, sizeof(int)) == cudaSuccess;
  if (!ok) return ICEP_ERR_CUDA;
  cudaMemsetAsync(err, 0, sizeof(int), s);
  // He-normal initial weights (zero biases), drawn on the host
  std::vector<float> h(nparams, 0.f);
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> nd(0.f, 1.f);
  for (int l = 0; l < L_COUNT; l++) {
    const float sd = std::sqrt(2.f / (27.f * cin[l]));
    for (long q = woff[l]; q < boff[l]; q++) h[q] = nd(rng) * sd;
  }
  cudaMemcpyAsync(params, h.data(), sizeof(float) * nparams, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(adam_m, 0, sizeof(float) * nparams, s);
  cudaMemsetAsync(adam_v, 0, sizeof(float) * nparams, s);
  adam_t = 0;
  pack(s);
  return cudaStreamSynchronize(s) == cudaSuccess ? ICEP_OK : ICEP_ERR_CUDA;
}

void UNet::free_all() {
  float *fs[] = {params, grads, adam_m, adam_v, x, y, gy, tmp, g0, g1};
  for (float *p : fs) cudaFree(p);
  bf16 *bs[] = {wf, wb, e0a, e0, p1, e1a, e1, p2, e2a, e2, d1, d0, gz, gz2};
  for (bf16 *p : bs) cudaFree(p);
  cudaFree(err);
  params = nullptr;
}

void UNet::pack(cudaStream_t s) {
  for (int l = L_C0B; l <= L_C0U; l++) {
    const int cnt = 27 * cin[l] * cout[l];
    count_launch();
    k_pack_layer<<<nb256(cnt), 256, 0, s>>>(cin[l], cout[l], params + woff[l], wf + wbf_off[l], wb + wbf_off[l]);
  }
}

void UNet::selftest_wait(cudaStream_t s) {
  conv_tc<16, 0, 16, true>(ilog2(n), e0a, nullptr, wf + wbf_off[L_C0B], params + boff[L_C0B], e0, err, s, 1);
}

void UNet::forward(cudaStream_t s) {
  const int lg = ilog2(n);
  const long V0 = (long)n * n * n, V1 = V0 / 8, V2 = V0 / 64;
  count_launch();
  k_conv_in<<<nb256(V0), 256, 0, s>>>(lg, x, params + woff[L_C0A], params + boff[L_C0A], e0a);
  conv_tc<16, 0, 16, true>(lg, e0a, nullptr, wf + wbf_off[L_C0B], params + boff[L_C0B], e0, err, s);
  count_launch();
  k_pool<<<nb256(V1 * 16), 256, 0, s>>>(lg, 16, e0, p1);
  conv_tc<16, 0, 32, true>(lg - 1, p1, nullptr, wf + wbf_off[L_C1A], params + boff[L_C1A], e1a, err, s);
  conv_tc<32, 0, 32, true>(lg - 1, e1a, nullptr, wf + wbf_off[L_C1B], params + boff[L_C1B], e1, err, s);
  count_launch();
  k_pool<<<nb256(V2 * 32), 256, 0, s>>>(lg - 1, 32, e1, p2);
  conv_tc<32, 0, 64, true>(lg - 2, p2, nullptr, wf + wbf_off[L_C2A], params + boff[L_C2A], e2a, err, s);
  conv_tc<64, 0, 64, true>(lg - 2, e2a, nullptr, wf + wbf_off[L_C2B], params + boff[L_C2B], e2, err, s);
  conv_tc<32, 64, 32, true>(lg - 1, e1, e2, wf + wbf_off[L_C1U], params + boff[L_C1U], d1, err, s);
  conv_tc<16, 32, 16, true>(lg, e0, d1, wf + wbf_off[L_C0U], params + boff[L_C0U], d0, err, s);
  count_launch();
  k_conv_out<<<nb256(V0), 256, 0, s>>>(lg, d0, params + woff[L_OUT], params + boff[L_OUT], y);
}

void UNet::backward(cudaStream_t s) {
  const int lg = ilog2(n);
  const long V0 = (long)n * n * n, V1 = V0 / 8, V2 = V0 / 64;
  float *G = grads;
  cudaMemsetAsync(grads, 0, sizeof(float) * nparams, s);
  // output layer
  conv_wgrad<bf16, float, 16, 0, 1>(lg, d0, nullptr, gy, G + woff[L_OUT], G + boff[L_OUT], s);
  count_launch();
  k_conv_out_bwd<<<nb256(V0), 256, 0, s>>>(lg, gy, params + woff[L_OUT], d0, gz);
  // c0u: in = cat(e0, up d1)
  conv_wgrad<bf16, bf16, 16, 32, 16>(lg, e0, d1, gz, G + woff[L_C0U], G + boff[L_C0U], s);
  conv_mma<16, 0, 48, true, false>(lg, gz, nullptr, wb + wbf_off[L_C0U], nullptr, tmp, s);
  count_launch();
  k_take_cols<<<nb256(V0 * 16), 256, 0, s>>>(V0, 48, 16, tmp, g0);
  count_launch();
  k_up_adjoint<<<nb256(V1 * 32), 256, 0, s>>>(lg, 48, 16, 32, tmp, g1);
  count_launch();
  k_relu_mask<<<nb256(V1 * 32), 256, 0, s>>>(V1 * 32, g1, d1, gz2);
  // c1u: in = cat(e1, up e2)
  conv_wgrad<bf16, bf16, 32, 64, 32>(lg - 1, e1, e2, gz2, G + woff[L_C1U], G + boff[L_C1U], s);
  conv_mma<32, 0, 96, true, false>(lg - 1, gz2, nullptr, wb + wbf_off[L_C1U], nullptr, tmp, s);
  count_launch();
  k_take_cols<<<nb256(V1 * 32), 256, 0, s>>>(V1, 96, 32, tmp, g1);
  float *g2 = tmp + 96 * V1;  // free space after the c1u gradient
  count_launch();
  k_up_adjoint<<<nb256(V2 * 64), 256, 0, s>>>(lg - 1, 96, 32, 64, tmp, g2);
  count_launch();
  k_relu_mask<<<nb256(V2 * 64), 256, 0, s>>>(V2 * 64, g2, e2, gz);
  // c2b, c2a
  conv_wgrad<bf16, bf16, 64, 0, 64>(lg - 2, e2a, nullptr, gz, G + woff[L_C2B], G + boff[L_C2B], s);
  conv_mma<64, 0, 64, true, false>(lg - 2, gz, nullptr, wb + wbf_off[L_C2B], nullptr, tmp, s);
  count_launch();
  k_relu_mask<<<nb256(V2 * 64), 256, 0, s>>>(V2 * 64, tmp, e2a, gz2);
  conv_wgrad<bf16, bf16, 32, 0, 64>(lg - 2, p2, nullptr, gz2, G + woff[L_C2A], G + boff[L_C2A], s);
  conv_mma<64, 0, 32, true, false>(lg - 2, gz2, nullptr, wb + wbf_off[L_C2A], nullptr, tmp, s);
  count_launch();
  k_pool_adjoint_add<<<nb256(V1 * 32), 256, 0, s>>>(lg - 1, 32, tmp, g1);
  count_launch();
  k_relu_mask<<<nb256(V1 * 32), 256, 0, s>>>(V1 * 32, g1, e1, gz);
  // c1b, c1a
  conv_wgrad<bf16, bf16, 32, 0, 32>(lg - 1, e1a, nullptr, gz, G + woff[L_C1B], G + boff[L_C1B], s);
  conv_mma<32, 0, 32, true, false>(lg - 1, gz, nullptr, wb + wbf_off[L_C1B], nullptr, tmp, s);
  count_launch();
  k_relu_mask<<<nb256(V1 * 32), 256, 0, s>>>(V1 * 32, tmp, e1a, gz2);
  conv_wgrad<bf16, bf16, 16, 0, 32>(lg - 1, p1, nullptr, gz2, G + woff[L_C1A], G + boff[L_C1A], s);
  conv_mma<32, 0, 16, true, false>(lg - 1, gz2, nullptr, wb + wbf_off[L_C1A], nullptr, tmp, s);
  count_launch();
  k_pool_adjoint_add<<<nb256(V0 * 16), 256, 0, s>>>(lg, 16, tmp, g0);
  count_launch();
  k_relu_mask<<<nb256(V0 * 16), 256, 0, s>>>(V0 * 16, g0, e0, gz);
  // c0b, c0a
  conv_wgrad<bf16, bf16, 16, 0, 16>(lg, e0a, nullptr, gz, G + woff[L_C0B], G + boff[L_C0B], s);
  conv_mma<16, 0, 16, true, false>(lg, gz, nullptr, wb + wbf_off[L_C0B], nullptr, tmp, s);
  count_launch();
  k_relu_mask<<<nb256(V0 * 16), 256, 0, s>>>(V0 * 16, tmp, e0a, gz2);
  conv_wgrad<float, bf16, 2, 0, 16>(lg, x, nullptr, gz2, G + woff[L_C0A], G + boff[L_C0A], s);
}

void UNet::adam_step(float lr, cudaStream_t s) {
  adam_t++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - powf(b1, (float)adam_t), bc2 = 1.f - powf(b2, (float)adam_t);
  count_launch();
  k_adam<<<nb256(nparams), 256, 0, s>>>(nparams, params, grads, adam_m, adam_v, lr, b1, b2, 1e-8f, bc1, bc2);
  pack(s);
}

void unet_input(const Grid &g, const float *eps, const float *r, double eps_ref, double rms, float *x, cudaStream_t s) {
  const int lgc = ilog2(g.nx / 2);
  count_launch();
  k_unet_input<<<nb256(1L << (3 * lgc)), 256, 0, s>>>(g, lgc, eps, r, (float)(1.0 / eps_ref),
                                                      (float)(rms > 0 ? 1.0 / rms : 1.0), x);
}

void unet_prolong_add(const Grid &g, const float *y, double scale, float *z, cudaStream_t s) {
  count_launch();
  k_prolong_add<<<nb256(g.nreal()), 256, 0, s>>>(g, ilog2(g.nx / 2), y, (float)scale, z);
}

void unet_prolong_adjoint(const Grid &g, const float *dz, double scale, float *gy, cudaStream_t s) {
  const int lgc = ilog2(g.nx / 2);
  count_launch();
  k_prolong_adjoint<<<nb256(1L << (3 * lgc)), 256, 0, s>>>(g, lgc, dz, (float)scale, gy);
}

}  // namespace icep
