// wave_c.cu -- wavefront kernel instantiations for K = 17, 18, 19, 20, 21, 22, 23, 24
// (split across files so the build compiles them in parallel).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_c(int K, int mode, int pair) {
  switch (K) {
    case 17:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<17, SG, true> : (WaveFn)wave_kernel<17, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<17, SW, true> : (WaveFn)wave_kernel<17, SW, false>);
    case 18:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<18, SG, true> : (WaveFn)wave_kernel<18, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<18, SW, true> : (WaveFn)wave_kernel<18, SW, false>);
    case 19:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<19, SG, true> : (WaveFn)wave_kernel<19, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<19, SW, true> : (WaveFn)wave_kernel<19, SW, false>);
    case 20:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<20, SG, true> : (WaveFn)wave_kernel<20, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<20, SW, true> : (WaveFn)wave_kernel<20, SW, false>);
    case 21:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<21, SG, true> : (WaveFn)wave_kernel<21, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<21, SW, true> : (WaveFn)wave_kernel<21, SW, false>);
    case 22:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<22, SG, true> : (WaveFn)wave_kernel<22, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<22, SW, true> : (WaveFn)wave_kernel<22, SW, false>);
    case 23:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<23, SG, true> : (WaveFn)wave_kernel<23, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<23, SW, true> : (WaveFn)wave_kernel<23, SW, false>);
    case 24:
      return mode == SG ? (pair ? (WaveFn)wave_kernel<24, SG, true> : (WaveFn)wave_kernel<24, SG, false>)
                        : (pair ? (WaveFn)wave_kernel<24, SW, true> : (WaveFn)wave_kernel<24, SW, false>);
    default:
      return nullptr;
  }
}

BatchFn batch_fn_c(int K, int mode, int pair) {
  switch (K) {
    case 17:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<17, SG, true> : (BatchFn)batch_kernel<17, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<17, SW, true> : (BatchFn)batch_kernel<17, SW, false>);
    case 18:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<18, SG, true> : (BatchFn)batch_kernel<18, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<18, SW, true> : (BatchFn)batch_kernel<18, SW, false>);
    case 19:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<19, SG, true> : (BatchFn)batch_kernel<19, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<19, SW, true> : (BatchFn)batch_kernel<19, SW, false>);
    case 20:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<20, SG, true> : (BatchFn)batch_kernel<20, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<20, SW, true> : (BatchFn)batch_kernel<20, SW, false>);
    case 21:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<21, SG, true> : (BatchFn)batch_kernel<21, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<21, SW, true> : (BatchFn)batch_kernel<21, SW, false>);
    case 22:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<22, SG, true> : (BatchFn)batch_kernel<22, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<22, SW, true> : (BatchFn)batch_kernel<22, SW, false>);
    case 23:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<23, SG, true> : (BatchFn)batch_kernel<23, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<23, SW, true> : (BatchFn)batch_kernel<23, SW, false>);
    case 24:
      return mode == SG ? (pair ? (BatchFn)batch_kernel<24, SG, true> : (BatchFn)batch_kernel<24, SG, false>)
                        : (pair ? (BatchFn)batch_kernel<24, SW, true> : (BatchFn)batch_kernel<24, SW, false>);
    default:
      return nullptr;
  }
}

}  // namespace ish
