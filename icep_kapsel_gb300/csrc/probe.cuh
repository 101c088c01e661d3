// probe.cuh -- per-launch device timing of one kernel class while a caller's
// timed region runs: CUDA events recorded on the launching stream right
// before and after every launch of the selected class, summed on stop.
#pragma once
#include "common.cuh"

namespace icep {

// Kernel classes that can be probed (values of icep_probe_start's kind).
enum ProbeKind {
  PROBE_NONE = 0,
  PROBE_KOP_PLANE = 1,  // fused plane pass of the k-space operator (3 components)
  PROBE_KOP_XINV = 2,   // fused inverse x pass (vector update + gradient)
  PROBE_KOP_XFWD = 3,   // fused forward x pass (divergence + dot partials)
};

extern int g_probe_kind;
void probe_record_begin(cudaStream_t s);
void probe_record_end(double bytes, cudaStream_t s);
inline void probe_begin(int kind, cudaStream_t s) {
  if (kind == g_probe_kind) probe_record_begin(s);
}
inline void probe_end(int kind, double bytes, cudaStream_t s) {
  if (kind == g_probe_kind) probe_record_end(bytes, s);
}

}  // namespace icep
