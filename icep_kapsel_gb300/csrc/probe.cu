// probe.cu -- see probe.cuh; the C entry points are icep_probe_start/stop.
#include <vector>

#include "probe.cuh"

namespace icep {

int g_probe_kind = PROBE_NONE;

namespace {
struct ProbeState {
  std::vector<cudaEvent_t> ev;  // begin/end pairs
  int used = 0;                 // events recorded
  long long launches = 0;       // launches seen (recorded or not)
  double bytes = 0.0;           // algorithmic bytes of the recorded launches
};
ProbeState g_probe;
}  // namespace

void probe_record_begin(cudaStream_t s) {
  ProbeState &p = g_probe;
  p.launches++;
  if (p.used + 2 > (int)p.ev.size()) return;
  cudaEventRecord(p.ev[p.used], s);
}

void probe_record_end(double bytes, cudaStream_t s) {
  ProbeState &p = g_probe;
  if (p.used + 2 > (int)p.ev.size()) return;
  cudaEventRecord(p.ev[p.used + 1], s);
  p.used += 2;
  p.bytes += bytes;
}

}  // namespace icep

extern "C" int icep_probe_start(int kind, int max_launches) {
  using namespace icep;
  if (kind < PROBE_KOP_PLANE || kind > PROBE_KOP_XFWD || max_launches <= 0) return ICEP_ERR_ARG;
  ProbeState &p = g_probe;
  for (cudaEvent_t e : p.ev) cudaEventDestroy(e);
  p = ProbeState();
  p.ev.resize(2 * (size_t)max_launches);
  for (auto &e : p.ev)
    if (cudaEventCreate(&e) != cudaSuccess) return ICEP_ERR_CUDA;
  g_probe_kind = kind;
  return ICEP_OK;
}

extern "C" int icep_probe_stop(double *ms_total, long long *launches_timed, double *bytes_total) {
  using namespace icep;
  ProbeState &p = g_probe;
  g_probe_kind = PROBE_NONE;
  double ms = 0.0;
  int st = ICEP_OK;
  for (int k = 0; k + 1 < p.used; k += 2) {
    float t = 0.f;
    if (cudaEventSynchronize(p.ev[k + 1]) != cudaSuccess || cudaEventElapsedTime(&t, p.ev[k], p.ev[k + 1]) != cudaSuccess) {
      st = ICEP_ERR_CUDA;
      break;
    }
    ms += t;
  }
  if (ms_total) *ms_total = ms;
  if (launches_timed) *launches_timed = p.used / 2;
  if (bytes_total) *bytes_total = p.bytes;
  for (cudaEvent_t e : p.ev) cudaEventDestroy(e);
  p = ProbeState();
  return st;
}
