// wave_f.cu -- wavefront kernel instantiations for K = 50, 52, 54, 56, 58, 60, 62, 64
// (split across files so the build compiles them in parallel).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_f(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 50: {
      static const WaveFn t[2][3] = {
          {wave_kernel<50, SG, PROF_S16>, wave_kernel<50, SG, PROF_PAIR>, wave_kernel<50, SG, PROF_S32>},
          {wave_kernel<50, SW, PROF_S16>, wave_kernel<50, SW, PROF_PAIR>, wave_kernel<50, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 52: {
      static const WaveFn t[2][3] = {
          {wave_kernel<52, SG, PROF_S16>, wave_kernel<52, SG, PROF_PAIR>, wave_kernel<52, SG, PROF_S32>},
          {wave_kernel<52, SW, PROF_S16>, wave_kernel<52, SW, PROF_PAIR>, wave_kernel<52, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 54: {
      static const WaveFn t[2][3] = {
          {wave_kernel<54, SG, PROF_S16>, wave_kernel<54, SG, PROF_PAIR>, wave_kernel<54, SG, PROF_S32>},
          {wave_kernel<54, SW, PROF_S16>, wave_kernel<54, SW, PROF_PAIR>, wave_kernel<54, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 56: {
      static const WaveFn t[2][3] = {
          {wave_kernel<56, SG, PROF_S16>, wave_kernel<56, SG, PROF_PAIR>, wave_kernel<56, SG, PROF_S32>},
          {wave_kernel<56, SW, PROF_S16>, wave_kernel<56, SW, PROF_PAIR>, wave_kernel<56, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 58: {
      static const WaveFn t[2][3] = {
          {wave_kernel<58, SG, PROF_S16>, wave_kernel<58, SG, PROF_PAIR>, wave_kernel<58, SG, PROF_S32>},
          {wave_kernel<58, SW, PROF_S16>, wave_kernel<58, SW, PROF_PAIR>, wave_kernel<58, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 60: {
      static const WaveFn t[2][3] = {
          {wave_kernel<60, SG, PROF_S16>, wave_kernel<60, SG, PROF_PAIR>, wave_kernel<60, SG, PROF_S32>},
          {wave_kernel<60, SW, PROF_S16>, wave_kernel<60, SW, PROF_PAIR>, wave_kernel<60, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 62: {
      static const WaveFn t[2][3] = {
          {wave_kernel<62, SG, PROF_S16>, wave_kernel<62, SG, PROF_PAIR>, wave_kernel<62, SG, PROF_S32>},
          {wave_kernel<62, SW, PROF_S16>, wave_kernel<62, SW, PROF_PAIR>, wave_kernel<62, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 64: {
      static const WaveFn t[2][3] = {
          {wave_kernel<64, SG, PROF_S16>, wave_kernel<64, SG, PROF_PAIR>, wave_kernel<64, SG, PROF_S32>},
          {wave_kernel<64, SW, PROF_S16>, wave_kernel<64, SW, PROF_PAIR>, wave_kernel<64, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

BatchFn batch_fn_f(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 50: {
      static const BatchFn t[2][3] = {
          {batch_kernel<50, SG, PROF_S16>, batch_kernel<50, SG, PROF_PAIR>, batch_kernel<50, SG, PROF_S32>},
          {batch_kernel<50, SW, PROF_S16>, batch_kernel<50, SW, PROF_PAIR>, batch_kernel<50, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 52: {
      static const BatchFn t[2][3] = {
          {batch_kernel<52, SG, PROF_S16>, batch_kernel<52, SG, PROF_PAIR>, batch_kernel<52, SG, PROF_S32>},
          {batch_kernel<52, SW, PROF_S16>, batch_kernel<52, SW, PROF_PAIR>, batch_kernel<52, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 54: {
      static const BatchFn t[2][3] = {
          {batch_kernel<54, SG, PROF_S16>, batch_kernel<54, SG, PROF_PAIR>, batch_kernel<54, SG, PROF_S32>},
          {batch_kernel<54, SW, PROF_S16>, batch_kernel<54, SW, PROF_PAIR>, batch_kernel<54, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 56: {
      static const BatchFn t[2][3] = {
          {batch_kernel<56, SG, PROF_S16>, batch_kernel<56, SG, PROF_PAIR>, batch_kernel<56, SG, PROF_S32>},
          {batch_kernel<56, SW, PROF_S16>, batch_kernel<56, SW, PROF_PAIR>, batch_kernel<56, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 58: {
      static const BatchFn t[2][3] = {
          {batch_kernel<58, SG, PROF_S16>, batch_kernel<58, SG, PROF_PAIR>, batch_kernel<58, SG, PROF_S32>},
          {batch_kernel<58, SW, PROF_S16>, batch_kernel<58, SW, PROF_PAIR>, batch_kernel<58, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 60: {
      static const BatchFn t[2][3] = {
          {batch_kernel<60, SG, PROF_S16>, batch_kernel<60, SG, PROF_PAIR>, batch_kernel<60, SG, PROF_S32>},
          {batch_kernel<60, SW, PROF_S16>, batch_kernel<60, SW, PROF_PAIR>, batch_kernel<60, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 62: {
      static const BatchFn t[2][3] = {
          {batch_kernel<62, SG, PROF_S16>, batch_kernel<62, SG, PROF_PAIR>, batch_kernel<62, SG, PROF_S32>},
          {batch_kernel<62, SW, PROF_S16>, batch_kernel<62, SW, PROF_PAIR>, batch_kernel<62, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 64: {
      static const BatchFn t[2][3] = {
          {batch_kernel<64, SG, PROF_S16>, batch_kernel<64, SG, PROF_PAIR>, batch_kernel<64, SG, PROF_S32>},
          {batch_kernel<64, SW, PROF_S16>, batch_kernel<64, SW, PROF_PAIR>, batch_kernel<64, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

}  // namespace ish
