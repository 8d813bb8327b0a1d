// wave_f.cu -- wavefront kernel instantiations for K = 50, 52, 54, 56, 58, 60, 62, 64
// (split across files so the build compiles them in parallel).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_f(int K, int mode, int pair) {
  switch (K) {
    case 50:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<50, SG, true> : (WaveFn)wave_kernel<50, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<50, SW, true> : (WaveFn)wave_kernel<50, SW, false>);
    case 52:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<52, SG, true> : (WaveFn)wave_kernel<52, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<52, SW, true> : (WaveFn)wave_kernel<52, SW, false>);
    case 54:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<54, SG, true> : (WaveFn)wave_kernel<54, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<54, SW, true> : (WaveFn)wave_kernel<54, SW, false>);
    case 56:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<56, SG, true> : (WaveFn)wave_kernel<56, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<56, SW, true> : (WaveFn)wave_kernel<56, SW, false>);
    case 58:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<58, SG, true> : (WaveFn)wave_kernel<58, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<58, SW, true> : (WaveFn)wave_kernel<58, SW, false>);
    case 60:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<60, SG, true> : (WaveFn)wave_kernel<60, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<60, SW, true> : (WaveFn)wave_kernel<60, SW, false>);
    case 62:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<62, SG, true> : (WaveFn)wave_kernel<62, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<62, SW, true> : (WaveFn)wave_kernel<62, SW, false>);
    case 64:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<64, SG, true> : (WaveFn)wave_kernel<64, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<64, SW, true> : (WaveFn)wave_kernel<64, SW, false>);
    default:
      return nullptr;
  }
}

BatchFn batch_fn_f(int K, int mode, int pair) {
  switch (K) {
    case 50:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<50, SG, true> : (BatchFn)batch_kernel<50, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<50, SW, true> : (BatchFn)batch_kernel<50, SW, false>);
    case 52:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<52, SG, true> : (BatchFn)batch_kernel<52, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<52, SW, true> : (BatchFn)batch_kernel<52, SW, false>);
    case 54:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<54, SG, true> : (BatchFn)batch_kernel<54, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<54, SW, true> : (BatchFn)batch_kernel<54, SW, false>);
    case 56:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<56, SG, true> : (BatchFn)batch_kernel<56, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<56, SW, true> : (BatchFn)batch_kernel<56, SW, false>);
    case 58:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<58, SG, true> : (BatchFn)batch_kernel<58, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<58, SW, true> : (BatchFn)batch_kernel<58, SW, false>);
    case 60:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<60, SG, true> : (BatchFn)batch_kernel<60, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<60, SW, true> : (BatchFn)batch_kernel<60, SW, false>);
    case 62:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<62, SG, true> : (BatchFn)batch_kernel<62, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<62, SW, true> : (BatchFn)batch_kernel<62, SW, false>);
    case 64:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<64, SG, true> : (BatchFn)batch_kernel<64, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<64, SW, true> : (BatchFn)batch_kernel<64, SW, false>);
    default:
      return nullptr;
  }
}

}  // namespace ish
