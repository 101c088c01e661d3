// unet.cuh -- the network of the learned Poisson preconditioner: a 3-level
// U-Net on the half-resolution grid (n = N/2 per axis), BF16 activations in
// channels-last layout, FP32 accumulation, periodic 3x3x3 convolutions.
//
//   input   x  = (eps_c/eps_ref - 1, r_c/rms(r))        2 ch,  n^3 (FP32)
//   level 0 e0 = relu(c0b(relu(c0a(x))))                16 ch, n^3
//   level 1 e1 = relu(c1b(relu(c1a(pool e0))))          32 ch, (n/2)^3
//   level 2 e2 = relu(c2b(relu(c2a(pool e1))))          64 ch, (n/4)^3
//   up 1    d1 = relu(c1u(cat(e1, up e2)))               32 ch, (n/2)^3
//   up 0    d0 = relu(c0u(cat(e0, up d1)))               16 ch, n^3
//   output  y  = out(d0)                                 1 ch,  n^3 (FP32)
//
// The 16..96-channel convolutions are implicit GEMMs on the tensor cores with
// FP32 accumulation: tcgen05.mma with a TMEM accumulator in the forward pass
// (inference and training), mma.sync for the data gradients of the backward
// pass; the 2-channel input and 1-channel output layers and the weight
// gradients run on the CUDA cores in FP32. The flat FP32 parameter vector and
// the tap/channel conventions are those of the CPU oracle (oracle/unet_ref.py).
#pragma once
#include <cuda_bf16.h>

#include "common.cuh"

namespace icep {

typedef __nv_bfloat16 bf16;

enum UNetLayer { L_C0A = 0, L_C0B, L_C1A, L_C1B, L_C2A, L_C2B, L_C1U, L_C0U, L_OUT, L_COUNT };

struct UNet {
  int n = 0;         // coarse grid edge (a power of two >= 16)
  long nparams = 0;  // FP32 parameters (weights + biases, oracle layout)
  long woff[L_COUNT], boff[L_COUNT];
  int cin[L_COUNT], cout[L_COUNT];
  float *params = nullptr, *grads = nullptr, *adam_m = nullptr, *adam_v = nullptr;
  bf16 *wf = nullptr, *wb = nullptr;  // BF16 weights: forward [t][co][ci]; backward-data [t][ci][co] (taps reversed)
  long wbf_off[L_COUNT];
  // activations
  float *x = nullptr, *y = nullptr;
  bf16 *e0a, *e0, *p1, *e1a, *e1, *p2, *e2a, *e2, *d1, *d0;
  // backward work
  float *gy = nullptr, *tmp = nullptr, *g0 = nullptr, *g1 = nullptr;
  bf16 *gz = nullptr, *gz2 = nullptr;
  int *err = nullptr;  // set by a tensor-core convolution whose completion wait ran out
  int adam_t = 0;

  int init(int n_coarse, unsigned long long seed, cudaStream_t s);
  void free_all();
  // refresh the BF16 weight copies from the FP32 parameters
  void pack(cudaStream_t s);
  // y = net(x) (x, y already filled / read by the caller)
  void forward(cudaStream_t s);
  // grads = dL/dparams given gy = dL/dy (forward() must have run on the same x)
  void backward(cudaStream_t s);
  void adam_step(float lr, cudaStream_t s);
  // one tcgen05 convolution launched so that its completion wait runs out
  // (no MMA is issued), which sets *err
  void selftest_wait(cudaStream_t s);
};

// x (coarse, 2 ch) from the fine permittivity and a fine real residual
// field (padded layout): (mean8(eps)/eps_ref - 1, mean8(r)/rms)
void unet_input(const Grid &g, const float *eps, const float *r, double eps_ref, double rms, float *x, cudaStream_t s);
// fine real field z += scale * prolong(y) (cell-centred trilinear, periodic)
void unet_prolong_add(const Grid &g, const float *y, double scale, float *z, cudaStream_t s);
// coarse gy = scale * prolong^T(dz) for a fine real field dz
void unet_prolong_adjoint(const Grid &g, const float *dz, double scale, float *gy, cudaStream_t s);

}  // namespace icep
