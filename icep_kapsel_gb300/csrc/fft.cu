// fft.cu -- the FFT kernels (fft_impl.cuh) for float and double.
#include "fft_impl.cuh"

namespace icep {

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
