// wave_b.cu -- wavefront kernel instantiations for K = 9, 10, 11, 12, 13, 14, 15, 16
// (split across files so the build compiles them in parallel).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_b(int K, int mode, int pair) {
  switch (K) {
    case 9:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<9, SG, true> : (WaveFn)wave_kernel<9, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<9, SW, true> : (WaveFn)wave_kernel<9, SW, false>);
    case 10:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<10, SG, true> : (WaveFn)wave_kernel<10, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<10, SW, true> : (WaveFn)wave_kernel<10, SW, false>);
    case 11:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<11, SG, true> : (WaveFn)wave_kernel<11, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<11, SW, true> : (WaveFn)wave_kernel<11, SW, false>);
    case 12:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<12, SG, true> : (WaveFn)wave_kernel<12, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<12, SW, true> : (WaveFn)wave_kernel<12, SW, false>);
    case 13:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<13, SG, true> : (WaveFn)wave_kernel<13, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<13, SW, true> : (WaveFn)wave_kernel<13, SW, false>);
    case 14:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<14, SG, true> : (WaveFn)wave_kernel<14, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<14, SW, true> : (WaveFn)wave_kernel<14, SW, false>);
    case 15:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<15, SG, true> : (WaveFn)wave_kernel<15, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<15, SW, true> : (WaveFn)wave_kernel<15, SW, false>);
    case 16:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<16, SG, true> : (WaveFn)wave_kernel<16, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<16, SW, true> : (WaveFn)wave_kernel<16, SW, false>);
    default:
      return nullptr;
  }
}

BatchFn batch_fn_b(int K, int mode, int pair) {
  switch (K) {
    case 9:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<9, SG, true> : (BatchFn)batch_kernel<9, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<9, SW, true> : (BatchFn)batch_kernel<9, SW, false>);
    case 10:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<10, SG, true> : (BatchFn)batch_kernel<10, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<10, SW, true> : (BatchFn)batch_kernel<10, SW, false>);
    case 11:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<11, SG, true> : (BatchFn)batch_kernel<11, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<11, SW, true> : (BatchFn)batch_kernel<11, SW, false>);
    case 12:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<12, SG, true> : (BatchFn)batch_kernel<12, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<12, SW, true> : (BatchFn)batch_kernel<12, SW, false>);
    case 13:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<13, SG, true> : (BatchFn)batch_kernel<13, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<13, SW, true> : (BatchFn)batch_kernel<13, SW, false>);
    case 14:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<14, SG, true> : (BatchFn)batch_kernel<14, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<14, SW, true> : (BatchFn)batch_kernel<14, SW, false>);
    case 15:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<15, SG, true> : (BatchFn)batch_kernel<15, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<15, SW, true> : (BatchFn)batch_kernel<15, SW, false>);
    case 16:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<16, SG, true> : (BatchFn)batch_kernel<16, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<16, SW, true> : (BatchFn)batch_kernel<16, SW, false>);
    default:
      return nullptr;
  }
}

}  // namespace ish
