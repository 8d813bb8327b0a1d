// wave_d.cu -- wavefront kernel instantiations for K = 25, 26, 27, 28, 29, 30, 31, 32
// (split across files so the build compiles them in parallel).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_d(int K, int mode, int pair) {
  switch (K) {
    case 25:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<25, SG, true> : (WaveFn)wave_kernel<25, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<25, SW, true> : (WaveFn)wave_kernel<25, SW, false>);
    case 26:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<26, SG, true> : (WaveFn)wave_kernel<26, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<26, SW, true> : (WaveFn)wave_kernel<26, SW, false>);
    case 27:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<27, SG, true> : (WaveFn)wave_kernel<27, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<27, SW, true> : (WaveFn)wave_kernel<27, SW, false>);
    case 28:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<28, SG, true> : (WaveFn)wave_kernel<28, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<28, SW, true> : (WaveFn)wave_kernel<28, SW, false>);
    case 29:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<29, SG, true> : (WaveFn)wave_kernel<29, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<29, SW, true> : (WaveFn)wave_kernel<29, SW, false>);
    case 30:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<30, SG, true> : (WaveFn)wave_kernel<30, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<30, SW, true> : (WaveFn)wave_kernel<30, SW, false>);
    case 31:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<31, SG, true> : (WaveFn)wave_kernel<31, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<31, SW, true> : (WaveFn)wave_kernel<31, SW, false>);
    case 32:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<32, SG, true> : (WaveFn)wave_kernel<32, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<32, SW, true> : (WaveFn)wave_kernel<32, SW, false>);
    default:
      return nullptr;
  }
}

BatchFn batch_fn_d(int K, int mode, int pair) {
  switch (K) {
    case 25:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<25, SG, true> : (BatchFn)batch_kernel<25, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<25, SW, true> : (BatchFn)batch_kernel<25, SW, false>);
    case 26:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<26, SG, true> : (BatchFn)batch_kernel<26, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<26, SW, true> : (BatchFn)batch_kernel<26, SW, false>);
    case 27:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<27, SG, true> : (BatchFn)batch_kernel<27, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<27, SW, true> : (BatchFn)batch_kernel<27, SW, false>);
    case 28:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<28, SG, true> : (BatchFn)batch_kernel<28, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<28, SW, true> : (BatchFn)batch_kernel<28, SW, false>);
    case 29:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<29, SG, true> : (BatchFn)batch_kernel<29, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<29, SW, true> : (BatchFn)batch_kernel<29, SW, false>);
    case 30:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<30, SG, true> : (BatchFn)batch_kernel<30, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<30, SW, true> : (BatchFn)batch_kernel<30, SW, false>);
    case 31:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<31, SG, true> : (BatchFn)batch_kernel<31, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<31, SW, true> : (BatchFn)batch_kernel<31, SW, false>);
    case 32:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<32, SG, true> : (BatchFn)batch_kernel<32, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<32, SW, true> : (BatchFn)batch_kernel<32, SW, false>);
    default:
      return nullptr;
  }
}

}  // namespace ish
