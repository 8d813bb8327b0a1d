// wave_b.cu -- wavefront kernel instantiations for K = 18..32
// (split across files so the build compiles them in parallel).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_b(int K, int mode, int pair) {
  switch (K) {
    case 18:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<18, SG, true> : (WaveFn)wave_kernel<18, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<18, SW, true> : (WaveFn)wave_kernel<18, SW, false>);
    case 20:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<20, SG, true> : (WaveFn)wave_kernel<20, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<20, SW, true> : (WaveFn)wave_kernel<20, SW, false>);
    case 22:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<22, SG, true> : (WaveFn)wave_kernel<22, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<22, SW, true> : (WaveFn)wave_kernel<22, SW, false>);
    case 24:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<24, SG, true> : (WaveFn)wave_kernel<24, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<24, SW, true> : (WaveFn)wave_kernel<24, SW, false>);
    case 26:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<26, SG, true> : (WaveFn)wave_kernel<26, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<26, SW, true> : (WaveFn)wave_kernel<26, SW, false>);
    case 28:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<28, SG, true> : (WaveFn)wave_kernel<28, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<28, SW, true> : (WaveFn)wave_kernel<28, SW, false>);
    case 30:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<30, SG, true> : (WaveFn)wave_kernel<30, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<30, SW, true> : (WaveFn)wave_kernel<30, SW, false>);
    case 32:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<32, SG, true> : (WaveFn)wave_kernel<32, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<32, SW, true> : (WaveFn)wave_kernel<32, SW, false>);
    default:
      return nullptr;
  }
}

}  // namespace ish
