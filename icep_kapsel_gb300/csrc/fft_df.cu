// fft_df.cu -- the FFT kernels (fft_impl.cuh) in float-float arithmetic
// (dfl, dfloat.cuh): the FP64-accurate transforms of the MIXED Poisson
// solve's residual, run on the FP32 pipes.
#include "fft_impl.cuh"

namespace icep {

template void fft_pass<dfl>(const FFTPlan<dfl> &, const FieldBatch<dfl> &, int, cudaStream_t);
template int fft_plan_init<dfl>(FFTPlan<dfl> &, const Grid &, cudaStream_t);
template void fft_plan_free<dfl>(FFTPlan<dfl> &);
template void fft_r2c<dfl>(const FFTPlan<dfl> &, const FieldBatch<dfl> &, cudaStream_t);
template void fft_c2r<dfl>(const FFTPlan<dfl> &, const FieldBatch<dfl> &, cudaStream_t);
template void fft_c2r_eps_r2c<dfl>(const FFTPlan<dfl> &, const FieldBatch<dfl> &, const float *, cudaStream_t);

}  // namespace icep
