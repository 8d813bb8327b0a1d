// wave_c.cu -- wavefront kernel instantiations for K = 17, 18, 19, 20, 21, 22, 23, 24
// (split across files so the build compiles them in parallel).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_c(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 17: {
      static const WaveFn t[2][3] = {
          {wave_kernel<17, SG, PROF_S16>, wave_kernel<17, SG, PROF_PAIR>, wave_kernel<17, SG, PROF_S32>},
          {wave_kernel<17, SW, PROF_S16>, wave_kernel<17, SW, PROF_PAIR>, wave_kernel<17, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 18: {
      static const WaveFn t[2][3] = {
          {wave_kernel<18, SG, PROF_S16>, wave_kernel<18, SG, PROF_PAIR>, wave_kernel<18, SG, PROF_S32>},
          {wave_kernel<18, SW, PROF_S16>, wave_kernel<18, SW, PROF_PAIR>, wave_kernel<18, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 19: {
      static const WaveFn t[2][3] = {
          {wave_kernel<19, SG, PROF_S16>, wave_kernel<19, SG, PROF_PAIR>, wave_kernel<19, SG, PROF_S32>},
          {wave_kernel<19, SW, PROF_S16>, wave_kernel<19, SW, PROF_PAIR>, wave_kernel<19, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 20: {
      static const WaveFn t[2][3] = {
          {wave_kernel<20, SG, PROF_S16>, wave_kernel<20, SG, PROF_PAIR>, wave_kernel<20, SG, PROF_S32>},
          {wave_kernel<20, SW, PROF_S16>, wave_kernel<20, SW, PROF_PAIR>, wave_kernel<20, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 21: {
      static const WaveFn t[2][3] = {
          {wave_kernel<21, SG, PROF_S16>, wave_kernel<21, SG, PROF_PAIR>, wave_kernel<21, SG, PROF_S32>},
          {wave_kernel<21, SW, PROF_S16>, wave_kernel<21, SW, PROF_PAIR>, wave_kernel<21, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 22: {
      static const WaveFn t[2][3] = {
          {wave_kernel<22, SG, PROF_S16>, wave_kernel<22, SG, PROF_PAIR>, wave_kernel<22, SG, PROF_S32>},
          {wave_kernel<22, SW, PROF_S16>, wave_kernel<22, SW, PROF_PAIR>, wave_kernel<22, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 23: {
      static const WaveFn t[2][3] = {
          {wave_kernel<23, SG, PROF_S16>, wave_kernel<23, SG, PROF_PAIR>, wave_kernel<23, SG, PROF_S32>},
          {wave_kernel<23, SW, PROF_S16>, wave_kernel<23, SW, PROF_PAIR>, wave_kernel<23, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 24: {
      static const WaveFn t[2][3] = {
          {wave_kernel<24, SG, PROF_S16>, wave_kernel<24, SG, PROF_PAIR>, wave_kernel<24, SG, PROF_S32>},
          {wave_kernel<24, SW, PROF_S16>, wave_kernel<24, SW, PROF_PAIR>, wave_kernel<24, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

BatchFn batch_fn_c(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 17: {
      static const BatchFn t[2][3] = {
          {batch_kernel<17, SG, PROF_S16>, batch_kernel<17, SG, PROF_PAIR>, batch_kernel<17, SG, PROF_S32>},
          {batch_kernel<17, SW, PROF_S16>, batch_kernel<17, SW, PROF_PAIR>, batch_kernel<17, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 18: {
      static const BatchFn t[2][3] = {
          {batch_kernel<18, SG, PROF_S16>, batch_kernel<18, SG, PROF_PAIR>, batch_kernel<18, SG, PROF_S32>},
          {batch_kernel<18, SW, PROF_S16>, batch_kernel<18, SW, PROF_PAIR>, batch_kernel<18, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 19: {
      static const BatchFn t[2][3] = {
          {batch_kernel<19, SG, PROF_S16>, batch_kernel<19, SG, PROF_PAIR>, batch_kernel<19, SG, PROF_S32>},
          {batch_kernel<19, SW, PROF_S16>, batch_kernel<19, SW, PROF_PAIR>, batch_kernel<19, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 20: {
      static const BatchFn t[2][3] = {
          {batch_kernel<20, SG, PROF_S16>, batch_kernel<20, SG, PROF_PAIR>, batch_kernel<20, SG, PROF_S32>},
          {batch_kernel<20, SW, PROF_S16>, batch_kernel<20, SW, PROF_PAIR>, batch_kernel<20, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 21: {
      static const BatchFn t[2][3] = {
          {batch_kernel<21, SG, PROF_S16>, batch_kernel<21, SG, PROF_PAIR>, batch_kernel<21, SG, PROF_S32>},
          {batch_kernel<21, SW, PROF_S16>, batch_kernel<21, SW, PROF_PAIR>, batch_kernel<21, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 22: {
      static const BatchFn t[2][3] = {
          {batch_kernel<22, SG, PROF_S16>, batch_kernel<22, SG, PROF_PAIR>, batch_kernel<22, SG, PROF_S32>},
          {batch_kernel<22, SW, PROF_S16>, batch_kernel<22, SW, PROF_PAIR>, batch_kernel<22, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 23: {
      static const BatchFn t[2][3] = {
          {batch_kernel<23, SG, PROF_S16>, batch_kernel<23, SG, PROF_PAIR>, batch_kernel<23, SG, PROF_S32>},
          {batch_kernel<23, SW, PROF_S16>, batch_kernel<23, SW, PROF_PAIR>, batch_kernel<23, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 24: {
      static const BatchFn t[2][3] = {
          {batch_kernel<24, SG, PROF_S16>, batch_kernel<24, SG, PROF_PAIR>, batch_kernel<24, SG, PROF_S32>},
          {batch_kernel<24, SW, PROF_S16>, batch_kernel<24, SW, PROF_PAIR>, batch_kernel<24, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

}  // namespace ish
