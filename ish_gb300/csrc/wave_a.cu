// wave_a.cu -- wavefront kernel instantiations for K = 2..16
// (split across files so the build compiles them in parallel).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_a(int K, int mode, int pair) {
  switch (K) {
    case 2:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<2, SG, true> : (WaveFn)wave_kernel<2, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<2, SW, true> : (WaveFn)wave_kernel<2, SW, false>);
    case 4:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<4, SG, true> : (WaveFn)wave_kernel<4, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<4, SW, true> : (WaveFn)wave_kernel<4, SW, false>);
    case 6:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<6, SG, true> : (WaveFn)wave_kernel<6, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<6, SW, true> : (WaveFn)wave_kernel<6, SW, false>);
    case 8:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<8, SG, true> : (WaveFn)wave_kernel<8, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<8, SW, true> : (WaveFn)wave_kernel<8, SW, false>);
    case 10:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<10, SG, true> : (WaveFn)wave_kernel<10, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<10, SW, true> : (WaveFn)wave_kernel<10, SW, false>);
    case 12:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<12, SG, true> : (WaveFn)wave_kernel<12, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<12, SW, true> : (WaveFn)wave_kernel<12, SW, false>);
    case 14:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<14, SG, true> : (WaveFn)wave_kernel<14, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<14, SW, true> : (WaveFn)wave_kernel<14, SW, false>);
    case 16:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<16, SG, true> : (WaveFn)wave_kernel<16, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<16, SW, true> : (WaveFn)wave_kernel<16, SW, false>);
    default:
      return nullptr;
  }
}

}  // namespace ish
