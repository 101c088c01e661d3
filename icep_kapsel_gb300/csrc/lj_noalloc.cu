// lj_noalloc.cu -- the Lennard-Jones force on a caller-owned device particle
// array, with its cell-list scratch in a fixed device array of this library
// instead of memory allocated per context or per call.
//
// Who needs it: a caller that keeps its particles in its own device memory
// and may not allocate while it steps -- a host loop with a fixed device
// memory budget, or one that must not take the device-wide synchronisation
// that cudaMalloc/cudaFree imply in the middle of a step. This entry point
// needs no context and calls no allocating routine.
//
// Limits: at most ICEP_LJ_NOALLOC_MAX_PARTICLES particles and at most
// 16^3 cells (meshes up to 256^3 in cells of 16 DX); larger inputs are
// rejected with ICEP_ERR_UNSUPPORTED. All calls in the process share the one
// scratch array (per device), which keeps what the last call left in it:
// calls that may overlap in time (on different streams or host threads) race
// on it and must be serialised by the caller.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "../../include/icep_gb300.h"
#include "particles.cuh"

namespace icep {
namespace {

constexpr int kMaxCells = 16 * 16 * 16;
// layout of lj_force's work: cell starts (cells+1), cell fill counters
// (cells+1), particle list (np)
constexpr int kScratchInts = 2 * (kMaxCells + 1) + ICEP_LJ_NOALLOC_MAX_PARTICLES;

__device__ __align__(256) int g_lj_scratch[kScratchInts];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
int *g_scratch_ptr[kMaxDevices] = {nullptr};

// Address of g_lj_scratch on the current device, looked up once per device.
int scratch_for_current_device(int **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return ICEP_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_lj_scratch) != cudaSuccess || !p) return ICEP_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<int *>(p);
  }
  *out = g_scratch_ptr[dev];
  return ICEP_OK;
}

__global__ void k_clear_fr(icep_particle *p, int n) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a < n)
    for (int d = 0; d < 3; d++) p[a].fr[d] = 0.0;
}

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

int reject(int code, const char *msg) {
  fprintf(stderr, "icep_Calc_f_Lennard_Jones_noalloc: %s\n", msg);
  return code;
}

}  // namespace
}  // namespace icep

extern "C" int icep_Calc_f_Lennard_Jones_noalloc(const icep_params *params, icep_particle *d_particles,
                                                 int n_particles, void *stream) {
  using namespace icep;
  if (!params || n_particles < 0 || (n_particles > 0 && !d_particles))
    return reject(ICEP_ERR_ARG, "null parameters/particles or negative particle count");
  if (n_particles > ICEP_LJ_NOALLOC_MAX_PARTICLES)
    return reject(ICEP_ERR_UNSUPPORTED, "more particles than ICEP_LJ_NOALLOC_MAX_PARTICLES (65536)");
  const int N[3] = {params->nx, params->ny, params->nz};
  for (int d = 0; d < 3; d++)
    if (!pow2(N[d]) || N[d] < 16 || N[d] > 256)
      return reject(ICEP_ERR_UNSUPPORTED, "mesh sizes must be powers of two in [16, 256]");
  if (!(params->dx > 0.0)) return reject(ICEP_ERR_ARG, "non-positive DX");
  if (n_particles == 0) return ICEP_OK;
  // an error left pending by the caller's earlier work is reported, not
  // taken over (and not cleared)
  if (cudaPeekAtLastError() != cudaSuccess)
    return reject(ICEP_ERR_CUDA, "a CUDA error is pending from earlier work");
  int *scratch = nullptr;
  if (scratch_for_current_device(&scratch) != ICEP_OK)
    return reject(ICEP_ERR_CUDA, "cannot look up the device scratch array");

  // the Lennard-Jones constants of Set_global_parameters (input.cxx:404-440),
  // as a context derives them
  PartParams pp;
  memset(&pp, 0, sizeof(pp));
  pp.dx = params->dx;
  pp.radius = params->a * params->dx;
  for (int d = 0; d < 3; d++) {
    pp.L[d] = N[d] * params->dx;
    pp.N[d] = N[d];
  }
  pp.np = n_particles;
  lj_params_from(*params, pp);

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // fr accumulates in the gather: it starts from zero. The cell counters in
  // the scratch are reset by the cell kernel itself on every call, and the
  // particle list is written in full before it is read, so nothing left in
  // the scratch by an earlier call is used.
  count_launch();
  k_clear_fr<<<div_up(n_particles, 128), 128, 0, s>>>(d_particles, n_particles);
  cudaError_t e = cudaGetLastError();  // nothing was pending: this is the launch's own status
  if (e != cudaSuccess) return reject(ICEP_ERR_CUDA, cudaGetErrorString(e));
  if (pp.lj_on) {
    const int st = lj_force(pp, d_particles, scratch, kScratchInts, nullptr, 0, nullptr, s);
    if (st != ICEP_OK) return reject(st, "cell list does not fit the scratch array");
    e = cudaGetLastError();
    if (e != cudaSuccess) return reject(ICEP_ERR_CUDA, cudaGetErrorString(e));
  }
  return ICEP_OK;
}
