// wave_e.cu -- wavefront kernel instantiations for K = 34, 36, 38, 40, 42, 44, 46, 48
// (split across files so the build compiles them in parallel).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_e(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 34: {
      static const WaveFn t[2][3] = {
          {wave_kernel<34, SG, PROF_S16>, wave_kernel<34, SG, PROF_PAIR>, wave_kernel<34, SG, PROF_S32>},
          {wave_kernel<34, SW, PROF_S16>, wave_kernel<34, SW, PROF_PAIR>, wave_kernel<34, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 36: {
      static const WaveFn t[2][3] = {
          {wave_kernel<36, SG, PROF_S16>, wave_kernel<36, SG, PROF_PAIR>, wave_kernel<36, SG, PROF_S32>},
          {wave_kernel<36, SW, PROF_S16>, wave_kernel<36, SW, PROF_PAIR>, wave_kernel<36, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 38: {
      static const WaveFn t[2][3] = {
          {wave_kernel<38, SG, PROF_S16>, wave_kernel<38, SG, PROF_PAIR>, wave_kernel<38, SG, PROF_S32>},
          {wave_kernel<38, SW, PROF_S16>, wave_kernel<38, SW, PROF_PAIR>, wave_kernel<38, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 40: {
      static const WaveFn t[2][3] = {
          {wave_kernel<40, SG, PROF_S16>, wave_kernel<40, SG, PROF_PAIR>, wave_kernel<40, SG, PROF_S32>},
          {wave_kernel<40, SW, PROF_S16>, wave_kernel<40, SW, PROF_PAIR>, wave_kernel<40, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 42: {
      static const WaveFn t[2][3] = {
          {wave_kernel<42, SG, PROF_S16>, wave_kernel<42, SG, PROF_PAIR>, wave_kernel<42, SG, PROF_S32>},
          {wave_kernel<42, SW, PROF_S16>, wave_kernel<42, SW, PROF_PAIR>, wave_kernel<42, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 44: {
      static const WaveFn t[2][3] = {
          {wave_kernel<44, SG, PROF_S16>, wave_kernel<44, SG, PROF_PAIR>, wave_kernel<44, SG, PROF_S32>},
          {wave_kernel<44, SW, PROF_S16>, wave_kernel<44, SW, PROF_PAIR>, wave_kernel<44, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 46: {
      static const WaveFn t[2][3] = {
          {wave_kernel<46, SG, PROF_S16>, wave_kernel<46, SG, PROF_PAIR>, wave_kernel<46, SG, PROF_S32>},
          {wave_kernel<46, SW, PROF_S16>, wave_kernel<46, SW, PROF_PAIR>, wave_kernel<46, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 48: {
      static const WaveFn t[2][3] = {
          {wave_kernel<48, SG, PROF_S16>, wave_kernel<48, SG, PROF_PAIR>, wave_kernel<48, SG, PROF_S32>},
          {wave_kernel<48, SW, PROF_S16>, wave_kernel<48, SW, PROF_PAIR>, wave_kernel<48, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

BatchFn batch_fn_e(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 34: {
      static const BatchFn t[2][3] = {
          {batch_kernel<34, SG, PROF_S16>, batch_kernel<34, SG, PROF_PAIR>, batch_kernel<34, SG, PROF_S32>},
          {batch_kernel<34, SW, PROF_S16>, batch_kernel<34, SW, PROF_PAIR>, batch_kernel<34, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 36: {
      static const BatchFn t[2][3] = {
          {batch_kernel<36, SG, PROF_S16>, batch_kernel<36, SG, PROF_PAIR>, batch_kernel<36, SG, PROF_S32>},
          {batch_kernel<36, SW, PROF_S16>, batch_kernel<36, SW, PROF_PAIR>, batch_kernel<36, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 38: {
      static const BatchFn t[2][3] = {
          {batch_kernel<38, SG, PROF_S16>, batch_kernel<38, SG, PROF_PAIR>, batch_kernel<38, SG, PROF_S32>},
          {batch_kernel<38, SW, PROF_S16>, batch_kernel<38, SW, PROF_PAIR>, batch_kernel<38, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 40: {
      static const BatchFn t[2][3] = {
          {batch_kernel<40, SG, PROF_S16>, batch_kernel<40, SG, PROF_PAIR>, batch_kernel<40, SG, PROF_S32>},
          {batch_kernel<40, SW, PROF_S16>, batch_kernel<40, SW, PROF_PAIR>, batch_kernel<40, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 42: {
      static const BatchFn t[2][3] = {
          {batch_kernel<42, SG, PROF_S16>, batch_kernel<42, SG, PROF_PAIR>, batch_kernel<42, SG, PROF_S32>},
          {batch_kernel<42, SW, PROF_S16>, batch_kernel<42, SW, PROF_PAIR>, batch_kernel<42, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 44: {
      static const BatchFn t[2][3] = {
          {batch_kernel<44, SG, PROF_S16>, batch_kernel<44, SG, PROF_PAIR>, batch_kernel<44, SG, PROF_S32>},
          {batch_kernel<44, SW, PROF_S16>, batch_kernel<44, SW, PROF_PAIR>, batch_kernel<44, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 46: {
      static const BatchFn t[2][3] = {
          {batch_kernel<46, SG, PROF_S16>, batch_kernel<46, SG, PROF_PAIR>, batch_kernel<46, SG, PROF_S32>},
          {batch_kernel<46, SW, PROF_S16>, batch_kernel<46, SW, PROF_PAIR>, batch_kernel<46, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 48: {
      static const BatchFn t[2][3] = {
          {batch_kernel<48, SG, PROF_S16>, batch_kernel<48, SG, PROF_PAIR>, batch_kernel<48, SG, PROF_S32>},
          {batch_kernel<48, SW, PROF_S16>, batch_kernel<48, SW, PROF_PAIR>, batch_kernel<48, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

}  // namespace ish
