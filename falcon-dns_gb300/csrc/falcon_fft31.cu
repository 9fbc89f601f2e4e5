// The nonlinear pass for FFT plans whose largest radix is 19 to 31 (or a generic prime)
// (falcon_fft.cuh, instantiated for MAXP = 31).
#include "falcon_fft.cuh"

namespace falcon {

cudaError_t init_dft_tables_31() { return init_tables_here(); }

cudaError_t launch_nonlin_31(const NonlinArgs& a, cudaStream_t s) { return launch_nonlin_t<31>(a, s); }

}  // namespace falcon
