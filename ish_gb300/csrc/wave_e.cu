// wave_e.cu -- wavefront kernel instantiations for K = 34, 36, 38, 40, 42, 44, 46, 48
// (split across files so the build compiles them in parallel).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_e(int K, int mode, int pair) {
  switch (K) {
    case 34:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<34, SG, true> : (WaveFn)wave_kernel<34, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<34, SW, true> : (WaveFn)wave_kernel<34, SW, false>);
    case 36:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<36, SG, true> : (WaveFn)wave_kernel<36, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<36, SW, true> : (WaveFn)wave_kernel<36, SW, false>);
    case 38:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<38, SG, true> : (WaveFn)wave_kernel<38, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<38, SW, true> : (WaveFn)wave_kernel<38, SW, false>);
    case 40:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<40, SG, true> : (WaveFn)wave_kernel<40, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<40, SW, true> : (WaveFn)wave_kernel<40, SW, false>);
    case 42:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<42, SG, true> : (WaveFn)wave_kernel<42, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<42, SW, true> : (WaveFn)wave_kernel<42, SW, false>);
    case 44:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<44, SG, true> : (WaveFn)wave_kernel<44, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<44, SW, true> : (WaveFn)wave_kernel<44, SW, false>);
    case 46:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<46, SG, true> : (WaveFn)wave_kernel<46, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<46, SW, true> : (WaveFn)wave_kernel<46, SW, false>);
    case 48:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<48, SG, true> : (WaveFn)wave_kernel<48, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<48, SW, true> : (WaveFn)wave_kernel<48, SW, false>);
    default:
      return nullptr;
  }
}

BatchFn batch_fn_e(int K, int mode, int pair) {
  switch (K) {
    case 34:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<34, SG, true> : (BatchFn)batch_kernel<34, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<34, SW, true> : (BatchFn)batch_kernel<34, SW, false>);
    case 36:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<36, SG, true> : (BatchFn)batch_kernel<36, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<36, SW, true> : (BatchFn)batch_kernel<36, SW, false>);
    case 38:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<38, SG, true> : (BatchFn)batch_kernel<38, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<38, SW, true> : (BatchFn)batch_kernel<38, SW, false>);
    case 40:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<40, SG, true> : (BatchFn)batch_kernel<40, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<40, SW, true> : (BatchFn)batch_kernel<40, SW, false>);
    case 42:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<42, SG, true> : (BatchFn)batch_kernel<42, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<42, SW, true> : (BatchFn)batch_kernel<42, SW, false>);
    case 44:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<44, SG, true> : (BatchFn)batch_kernel<44, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<44, SW, true> : (BatchFn)batch_kernel<44, SW, false>);
    case 46:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<46, SG, true> : (BatchFn)batch_kernel<46, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<46, SW, true> : (BatchFn)batch_kernel<46, SW, false>);
    case 48:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<48, SG, true> : (BatchFn)batch_kernel<48, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<48, SW, true> : (BatchFn)batch_kernel<48, SW, false>);
    default:
      return nullptr;
  }
}

}  // namespace ish
