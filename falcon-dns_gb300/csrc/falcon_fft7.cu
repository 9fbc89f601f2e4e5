// The nonlinear pass for FFT plans whose largest radix is at most 7
// (falcon_fft.cuh, instantiated for MAXP = 7).
#include "falcon_fft.cuh"

namespace falcon {

cudaError_t init_dft_tables_7() { return init_tables_here(); }

cudaError_t launch_nonlin_7(const NonlinArgs& a, cudaStream_t s) { return launch_nonlin_t<7>(a, s); }

}  // namespace falcon
