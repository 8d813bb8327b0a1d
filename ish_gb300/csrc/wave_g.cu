// wave_g.cu -- lean (128 x 2) wavefront kernel instantiations for K = 34, 36, 38, 40, 42, 44, 46, 48
// (see wave_blocks_lean in kernels.cuh).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_g(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 34: {
      static const WaveFn t[2][3] = {
          {wave_kernel<34, SG, PROF_S16, 1>, wave_kernel<34, SG, PROF_PAIR, 1>, wave_kernel<34, SG, PROF_S32, 1>},
          {wave_kernel<34, SW, PROF_S16, 1>, wave_kernel<34, SW, PROF_PAIR, 1>, wave_kernel<34, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 36: {
      static const WaveFn t[2][3] = {
          {wave_kernel<36, SG, PROF_S16, 1>, wave_kernel<36, SG, PROF_PAIR, 1>, wave_kernel<36, SG, PROF_S32, 1>},
          {wave_kernel<36, SW, PROF_S16, 1>, wave_kernel<36, SW, PROF_PAIR, 1>, wave_kernel<36, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 38: {
      static const WaveFn t[2][3] = {
          {wave_kernel<38, SG, PROF_S16, 1>, wave_kernel<38, SG, PROF_PAIR, 1>, wave_kernel<38, SG, PROF_S32, 1>},
          {wave_kernel<38, SW, PROF_S16, 1>, wave_kernel<38, SW, PROF_PAIR, 1>, wave_kernel<38, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 40: {
      static const WaveFn t[2][3] = {
          {wave_kernel<40, SG, PROF_S16, 1>, wave_kernel<40, SG, PROF_PAIR, 1>, wave_kernel<40, SG, PROF_S32, 1>},
          {wave_kernel<40, SW, PROF_S16, 1>, wave_kernel<40, SW, PROF_PAIR, 1>, wave_kernel<40, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 42: {
      static const WaveFn t[2][3] = {
          {wave_kernel<42, SG, PROF_S16, 1>, wave_kernel<42, SG, PROF_PAIR, 1>, wave_kernel<42, SG, PROF_S32, 1>},
          {wave_kernel<42, SW, PROF_S16, 1>, wave_kernel<42, SW, PROF_PAIR, 1>, wave_kernel<42, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 44: {
      static const WaveFn t[2][3] = {
          {wave_kernel<44, SG, PROF_S16, 1>, wave_kernel<44, SG, PROF_PAIR, 1>, wave_kernel<44, SG, PROF_S32, 1>},
          {wave_kernel<44, SW, PROF_S16, 1>, wave_kernel<44, SW, PROF_PAIR, 1>, wave_kernel<44, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 46: {
      static const WaveFn t[2][3] = {
          {wave_kernel<46, SG, PROF_S16, 1>, wave_kernel<46, SG, PROF_PAIR, 1>, wave_kernel<46, SG, PROF_S32, 1>},
          {wave_kernel<46, SW, PROF_S16, 1>, wave_kernel<46, SW, PROF_PAIR, 1>, wave_kernel<46, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 48: {
      static const WaveFn t[2][3] = {
          {wave_kernel<48, SG, PROF_S16, 1>, wave_kernel<48, SG, PROF_PAIR, 1>, wave_kernel<48, SG, PROF_S32, 1>},
          {wave_kernel<48, SW, PROF_S16, 1>, wave_kernel<48, SW, PROF_PAIR, 1>, wave_kernel<48, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

BatchFn batch_fn_g(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 34: {
      static const BatchFn t[2][3] = {
          {batch_kernel<34, SG, PROF_S16, 1>, batch_kernel<34, SG, PROF_PAIR, 1>, batch_kernel<34, SG, PROF_S32, 1>},
          {batch_kernel<34, SW, PROF_S16, 1>, batch_kernel<34, SW, PROF_PAIR, 1>, batch_kernel<34, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 36: {
      static const BatchFn t[2][3] = {
          {batch_kernel<36, SG, PROF_S16, 1>, batch_kernel<36, SG, PROF_PAIR, 1>, batch_kernel<36, SG, PROF_S32, 1>},
          {batch_kernel<36, SW, PROF_S16, 1>, batch_kernel<36, SW, PROF_PAIR, 1>, batch_kernel<36, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 38: {
      static const BatchFn t[2][3] = {
          {batch_kernel<38, SG, PROF_S16, 1>, batch_kernel<38, SG, PROF_PAIR, 1>, batch_kernel<38, SG, PROF_S32, 1>},
          {batch_kernel<38, SW, PROF_S16, 1>, batch_kernel<38, SW, PROF_PAIR, 1>, batch_kernel<38, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 40: {
      static const BatchFn t[2][3] = {
          {batch_kernel<40, SG, PROF_S16, 1>, batch_kernel<40, SG, PROF_PAIR, 1>, batch_kernel<40, SG, PROF_S32, 1>},
          {batch_kernel<40, SW, PROF_S16, 1>, batch_kernel<40, SW, PROF_PAIR, 1>, batch_kernel<40, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 42: {
      static const BatchFn t[2][3] = {
          {batch_kernel<42, SG, PROF_S16, 1>, batch_kernel<42, SG, PROF_PAIR, 1>, batch_kernel<42, SG, PROF_S32, 1>},
          {batch_kernel<42, SW, PROF_S16, 1>, batch_kernel<42, SW, PROF_PAIR, 1>, batch_kernel<42, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 44: {
      static const BatchFn t[2][3] = {
          {batch_kernel<44, SG, PROF_S16, 1>, batch_kernel<44, SG, PROF_PAIR, 1>, batch_kernel<44, SG, PROF_S32, 1>},
          {batch_kernel<44, SW, PROF_S16, 1>, batch_kernel<44, SW, PROF_PAIR, 1>, batch_kernel<44, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 46: {
      static const BatchFn t[2][3] = {
          {batch_kernel<46, SG, PROF_S16, 1>, batch_kernel<46, SG, PROF_PAIR, 1>, batch_kernel<46, SG, PROF_S32, 1>},
          {batch_kernel<46, SW, PROF_S16, 1>, batch_kernel<46, SW, PROF_PAIR, 1>, batch_kernel<46, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 48: {
      static const BatchFn t[2][3] = {
          {batch_kernel<48, SG, PROF_S16, 1>, batch_kernel<48, SG, PROF_PAIR, 1>, batch_kernel<48, SG, PROF_S32, 1>},
          {batch_kernel<48, SW, PROF_S16, 1>, batch_kernel<48, SW, PROF_PAIR, 1>, batch_kernel<48, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

}  // namespace ish
