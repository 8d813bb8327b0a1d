// wave_a.cu -- wavefront kernel instantiations for K = 1, 2, 3, 4, 5, 6, 7, 8
// (split across files so the build compiles them in parallel).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_a(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 1: {
      static const WaveFn t[2][3] = {
          {wave_kernel<1, SG, PROF_S16>, wave_kernel<1, SG, PROF_PAIR>, wave_kernel<1, SG, PROF_S32>},
          {wave_kernel<1, SW, PROF_S16>, wave_kernel<1, SW, PROF_PAIR>, wave_kernel<1, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 2: {
      static const WaveFn t[2][3] = {
          {wave_kernel<2, SG, PROF_S16>, wave_kernel<2, SG, PROF_PAIR>, wave_kernel<2, SG, PROF_S32>},
          {wave_kernel<2, SW, PROF_S16>, wave_kernel<2, SW, PROF_PAIR>, wave_kernel<2, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 3: {
      static const WaveFn t[2][3] = {
          {wave_kernel<3, SG, PROF_S16>, wave_kernel<3, SG, PROF_PAIR>, wave_kernel<3, SG, PROF_S32>},
          {wave_kernel<3, SW, PROF_S16>, wave_kernel<3, SW, PROF_PAIR>, wave_kernel<3, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 4: {
      static const WaveFn t[2][3] = {
          {wave_kernel<4, SG, PROF_S16>, wave_kernel<4, SG, PROF_PAIR>, wave_kernel<4, SG, PROF_S32>},
          {wave_kernel<4, SW, PROF_S16>, wave_kernel<4, SW, PROF_PAIR>, wave_kernel<4, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 5: {
      static const WaveFn t[2][3] = {
          {wave_kernel<5, SG, PROF_S16>, wave_kernel<5, SG, PROF_PAIR>, wave_kernel<5, SG, PROF_S32>},
          {wave_kernel<5, SW, PROF_S16>, wave_kernel<5, SW, PROF_PAIR>, wave_kernel<5, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 6: {
      static const WaveFn t[2][3] = {
          {wave_kernel<6, SG, PROF_S16>, wave_kernel<6, SG, PROF_PAIR>, wave_kernel<6, SG, PROF_S32>},
          {wave_kernel<6, SW, PROF_S16>, wave_kernel<6, SW, PROF_PAIR>, wave_kernel<6, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 7: {
      static const WaveFn t[2][3] = {
          {wave_kernel<7, SG, PROF_S16>, wave_kernel<7, SG, PROF_PAIR>, wave_kernel<7, SG, PROF_S32>},
          {wave_kernel<7, SW, PROF_S16>, wave_kernel<7, SW, PROF_PAIR>, wave_kernel<7, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 8: {
      static const WaveFn t[2][3] = {
          {wave_kernel<8, SG, PROF_S16>, wave_kernel<8, SG, PROF_PAIR>, wave_kernel<8, SG, PROF_S32>},
          {wave_kernel<8, SW, PROF_S16>, wave_kernel<8, SW, PROF_PAIR>, wave_kernel<8, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

BatchFn batch_fn_a(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 1: {
      static const BatchFn t[2][3] = {
          {batch_kernel<1, SG, PROF_S16>, batch_kernel<1, SG, PROF_PAIR>, batch_kernel<1, SG, PROF_S32>},
          {batch_kernel<1, SW, PROF_S16>, batch_kernel<1, SW, PROF_PAIR>, batch_kernel<1, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 2: {
      static const BatchFn t[2][3] = {
          {batch_kernel<2, SG, PROF_S16>, batch_kernel<2, SG, PROF_PAIR>, batch_kernel<2, SG, PROF_S32>},
          {batch_kernel<2, SW, PROF_S16>, batch_kernel<2, SW, PROF_PAIR>, batch_kernel<2, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 3: {
      static const BatchFn t[2][3] = {
          {batch_kernel<3, SG, PROF_S16>, batch_kernel<3, SG, PROF_PAIR>, batch_kernel<3, SG, PROF_S32>},
          {batch_kernel<3, SW, PROF_S16>, batch_kernel<3, SW, PROF_PAIR>, batch_kernel<3, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 4: {
      static const BatchFn t[2][3] = {
          {batch_kernel<4, SG, PROF_S16>, batch_kernel<4, SG, PROF_PAIR>, batch_kernel<4, SG, PROF_S32>},
          {batch_kernel<4, SW, PROF_S16>, batch_kernel<4, SW, PROF_PAIR>, batch_kernel<4, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 5: {
      static const BatchFn t[2][3] = {
          {batch_kernel<5, SG, PROF_S16>, batch_kernel<5, SG, PROF_PAIR>, batch_kernel<5, SG, PROF_S32>},
          {batch_kernel<5, SW, PROF_S16>, batch_kernel<5, SW, PROF_PAIR>, batch_kernel<5, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 6: {
      static const BatchFn t[2][3] = {
          {batch_kernel<6, SG, PROF_S16>, batch_kernel<6, SG, PROF_PAIR>, batch_kernel<6, SG, PROF_S32>},
          {batch_kernel<6, SW, PROF_S16>, batch_kernel<6, SW, PROF_PAIR>, batch_kernel<6, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 7: {
      static const BatchFn t[2][3] = {
          {batch_kernel<7, SG, PROF_S16>, batch_kernel<7, SG, PROF_PAIR>, batch_kernel<7, SG, PROF_S32>},
          {batch_kernel<7, SW, PROF_S16>, batch_kernel<7, SW, PROF_PAIR>, batch_kernel<7, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 8: {
      static const BatchFn t[2][3] = {
          {batch_kernel<8, SG, PROF_S16>, batch_kernel<8, SG, PROF_PAIR>, batch_kernel<8, SG, PROF_S32>},
          {batch_kernel<8, SW, PROF_S16>, batch_kernel<8, SW, PROF_PAIR>, batch_kernel<8, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

}  // namespace ish
