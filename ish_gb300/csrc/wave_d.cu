// wave_d.cu -- wavefront kernel instantiations for K = 25, 26, 27, 28, 29, 30, 31, 32
// (split across files so the build compiles them in parallel).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_d(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 25: {
      static const WaveFn t[2][3] = {
          {wave_kernel<25, SG, PROF_S16>, wave_kernel<25, SG, PROF_PAIR>, wave_kernel<25, SG, PROF_S32>},
          {wave_kernel<25, SW, PROF_S16>, wave_kernel<25, SW, PROF_PAIR>, wave_kernel<25, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 26: {
      static const WaveFn t[2][3] = {
          {wave_kernel<26, SG, PROF_S16>, wave_kernel<26, SG, PROF_PAIR>, wave_kernel<26, SG, PROF_S32>},
          {wave_kernel<26, SW, PROF_S16>, wave_kernel<26, SW, PROF_PAIR>, wave_kernel<26, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 27: {
      static const WaveFn t[2][3] = {
          {wave_kernel<27, SG, PROF_S16>, wave_kernel<27, SG, PROF_PAIR>, wave_kernel<27, SG, PROF_S32>},
          {wave_kernel<27, SW, PROF_S16>, wave_kernel<27, SW, PROF_PAIR>, wave_kernel<27, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 28: {
      static const WaveFn t[2][3] = {
          {wave_kernel<28, SG, PROF_S16>, wave_kernel<28, SG, PROF_PAIR>, wave_kernel<28, SG, PROF_S32>},
          {wave_kernel<28, SW, PROF_S16>, wave_kernel<28, SW, PROF_PAIR>, wave_kernel<28, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 29: {
      static const WaveFn t[2][3] = {
          {wave_kernel<29, SG, PROF_S16>, wave_kernel<29, SG, PROF_PAIR>, wave_kernel<29, SG, PROF_S32>},
          {wave_kernel<29, SW, PROF_S16>, wave_kernel<29, SW, PROF_PAIR>, wave_kernel<29, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 30: {
      static const WaveFn t[2][3] = {
          {wave_kernel<30, SG, PROF_S16>, wave_kernel<30, SG, PROF_PAIR>, wave_kernel<30, SG, PROF_S32>},
          {wave_kernel<30, SW, PROF_S16>, wave_kernel<30, SW, PROF_PAIR>, wave_kernel<30, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 31: {
      static const WaveFn t[2][3] = {
          {wave_kernel<31, SG, PROF_S16>, wave_kernel<31, SG, PROF_PAIR>, wave_kernel<31, SG, PROF_S32>},
          {wave_kernel<31, SW, PROF_S16>, wave_kernel<31, SW, PROF_PAIR>, wave_kernel<31, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 32: {
      static const WaveFn t[2][3] = {
          {wave_kernel<32, SG, PROF_S16>, wave_kernel<32, SG, PROF_PAIR>, wave_kernel<32, SG, PROF_S32>},
          {wave_kernel<32, SW, PROF_S16>, wave_kernel<32, SW, PROF_PAIR>, wave_kernel<32, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

BatchFn batch_fn_d(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 25: {
      static const BatchFn t[2][3] = {
          {batch_kernel<25, SG, PROF_S16>, batch_kernel<25, SG, PROF_PAIR>, batch_kernel<25, SG, PROF_S32>},
          {batch_kernel<25, SW, PROF_S16>, batch_kernel<25, SW, PROF_PAIR>, batch_kernel<25, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 26: {
      static const BatchFn t[2][3] = {
          {batch_kernel<26, SG, PROF_S16>, batch_kernel<26, SG, PROF_PAIR>, batch_kernel<26, SG, PROF_S32>},
          {batch_kernel<26, SW, PROF_S16>, batch_kernel<26, SW, PROF_PAIR>, batch_kernel<26, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 27: {
      static const BatchFn t[2][3] = {
          {batch_kernel<27, SG, PROF_S16>, batch_kernel<27, SG, PROF_PAIR>, batch_kernel<27, SG, PROF_S32>},
          {batch_kernel<27, SW, PROF_S16>, batch_kernel<27, SW, PROF_PAIR>, batch_kernel<27, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 28: {
      static const BatchFn t[2][3] = {
          {batch_kernel<28, SG, PROF_S16>, batch_kernel<28, SG, PROF_PAIR>, batch_kernel<28, SG, PROF_S32>},
          {batch_kernel<28, SW, PROF_S16>, batch_kernel<28, SW, PROF_PAIR>, batch_kernel<28, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 29: {
      static const BatchFn t[2][3] = {
          {batch_kernel<29, SG, PROF_S16>, batch_kernel<29, SG, PROF_PAIR>, batch_kernel<29, SG, PROF_S32>},
          {batch_kernel<29, SW, PROF_S16>, batch_kernel<29, SW, PROF_PAIR>, batch_kernel<29, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 30: {
      static const BatchFn t[2][3] = {
          {batch_kernel<30, SG, PROF_S16>, batch_kernel<30, SG, PROF_PAIR>, batch_kernel<30, SG, PROF_S32>},
          {batch_kernel<30, SW, PROF_S16>, batch_kernel<30, SW, PROF_PAIR>, batch_kernel<30, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 31: {
      static const BatchFn t[2][3] = {
          {batch_kernel<31, SG, PROF_S16>, batch_kernel<31, SG, PROF_PAIR>, batch_kernel<31, SG, PROF_S32>},
          {batch_kernel<31, SW, PROF_S16>, batch_kernel<31, SW, PROF_PAIR>, batch_kernel<31, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 32: {
      static const BatchFn t[2][3] = {
          {batch_kernel<32, SG, PROF_S16>, batch_kernel<32, SG, PROF_PAIR>, batch_kernel<32, SG, PROF_S32>},
          {batch_kernel<32, SW, PROF_S16>, batch_kernel<32, SW, PROF_PAIR>, batch_kernel<32, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

}  // namespace ish
