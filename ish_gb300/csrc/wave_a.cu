// wave_a.cu -- wavefront kernel instantiations for K = 1, 2, 3, 4, 5, 6, 7, 8
// (split across files so the build compiles them in parallel).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_a(int K, int mode, int pair) {
  switch (K) {
    case 1:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<1, SG, true> : (WaveFn)wave_kernel<1, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<1, SW, true> : (WaveFn)wave_kernel<1, SW, false>);
    case 2:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<2, SG, true> : (WaveFn)wave_kernel<2, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<2, SW, true> : (WaveFn)wave_kernel<2, SW, false>);
    case 3:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<3, SG, true> : (WaveFn)wave_kernel<3, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<3, SW, true> : (WaveFn)wave_kernel<3, SW, false>);
    case 4:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<4, SG, true> : (WaveFn)wave_kernel<4, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<4, SW, true> : (WaveFn)wave_kernel<4, SW, false>);
    case 5:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<5, SG, true> : (WaveFn)wave_kernel<5, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<5, SW, true> : (WaveFn)wave_kernel<5, SW, false>);
    case 6:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<6, SG, true> : (WaveFn)wave_kernel<6, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<6, SW, true> : (WaveFn)wave_kernel<6, SW, false>);
    case 7:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<7, SG, true> : (WaveFn)wave_kernel<7, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<7, SW, true> : (WaveFn)wave_kernel<7, SW, false>);
    case 8:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<8, SG, true> : (WaveFn)wave_kernel<8, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<8, SW, true> : (WaveFn)wave_kernel<8, SW, false>);
    default:
      return nullptr;
  }
}

BatchFn batch_fn_a(int K, int mode, int pair) {
  switch (K) {
    case 1:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<1, SG, true> : (BatchFn)batch_kernel<1, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<1, SW, true> : (BatchFn)batch_kernel<1, SW, false>);
    case 2:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<2, SG, true> : (BatchFn)batch_kernel<2, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<2, SW, true> : (BatchFn)batch_kernel<2, SW, false>);
    case 3:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<3, SG, true> : (BatchFn)batch_kernel<3, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<3, SW, true> : (BatchFn)batch_kernel<3, SW, false>);
    case 4:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<4, SG, true> : (BatchFn)batch_kernel<4, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<4, SW, true> : (BatchFn)batch_kernel<4, SW, false>);
    case 5:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<5, SG, true> : (BatchFn)batch_kernel<5, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<5, SW, true> : (BatchFn)batch_kernel<5, SW, false>);
    case 6:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<6, SG, true> : (BatchFn)batch_kernel<6, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<6, SW, true> : (BatchFn)batch_kernel<6, SW, false>);
    case 7:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<7, SG, true> : (BatchFn)batch_kernel<7, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<7, SW, true> : (BatchFn)batch_kernel<7, SW, false>);
    case 8:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<8, SG, true> : (BatchFn)batch_kernel<8, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<8, SW, true> : (BatchFn)batch_kernel<8, SW, false>);
    default:
      return nullptr;
  }
}

}  // namespace ish
