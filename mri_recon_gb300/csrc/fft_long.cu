// FFT passes for lines of 400..768 points (the default oversampled size of N = 257..512),
// 16 threads per line and a Q-point DFT of Q = S / 16 in registers (kernels in
// fft_kernels.cuh).  Q whose largest prime factor is above 23 (S = 464, 496, 592, 656,
// 688, 752) are not built.
#include "fft_kernels.cuh"

namespace mrg {

mrg_status launch_fft_long(const FftPass &p, cudaStream_t st) {
  switch (p.S) {
    case 400: return launch_q<25, 16>(p, st);
    case 416: return launch_q<26, 16>(p, st);
    case 432: return launch_q<27, 16>(p, st);
    case 448: return launch_q<28, 16>(p, st);
    case 480: return launch_q<30, 16>(p, st);
    case 512: return launch_q<32, 16>(p, st);
    case 528: return launch_q<33, 16>(p, st);
    case 544: return launch_q<34, 16>(p, st);
    case 560: return launch_q<35, 16>(p, st);
    case 576: return launch_q<36, 16>(p, st);
    case 608: return launch_q<38, 16>(p, st);
    case 624: return launch_q<39, 16>(p, st);
    case 640: return launch_q<40, 16>(p, st);
    case 672: return launch_q<42, 16>(p, st);
    case 704: return launch_q<44, 16>(p, st);
    case 720: return launch_q<45, 16>(p, st);
    case 736: return launch_q<46, 16>(p, st);
    case 768: return launch_q<48, 16>(p, st);
    default:
      set_error("unsupported FFT length " + std::to_string(p.S));
      return MRG_ERR_UNSUPPORTED;
  }
}

}  // namespace mrg
