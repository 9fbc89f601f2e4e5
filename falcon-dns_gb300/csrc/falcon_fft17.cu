// The nonlinear pass for FFT plans whose largest radix is 8 to 17
// (falcon_fft.cuh, instantiated for MAXP = 17).
#include "falcon_fft.cuh"

namespace falcon {

cudaError_t init_dft_tables_17() { return init_tables_here(); }

cudaError_t launch_nonlin_17(const NonlinArgs& a, cudaStream_t s) { return launch_nonlin_t<17>(a, s); }

}  // namespace falcon
