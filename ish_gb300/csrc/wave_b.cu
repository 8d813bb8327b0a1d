// wave_b.cu -- wavefront kernel instantiations for K = 9, 10, 11, 12, 13, 14, 15, 16
// (split across files so the build compiles them in parallel).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_b(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 9: {
      static const WaveFn t[2][3] = {
          {wave_kernel<9, SG, PROF_S16>, wave_kernel<9, SG, PROF_PAIR>, wave_kernel<9, SG, PROF_S32>},
          {wave_kernel<9, SW, PROF_S16>, wave_kernel<9, SW, PROF_PAIR>, wave_kernel<9, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 10: {
      static const WaveFn t[2][3] = {
          {wave_kernel<10, SG, PROF_S16>, wave_kernel<10, SG, PROF_PAIR>, wave_kernel<10, SG, PROF_S32>},
          {wave_kernel<10, SW, PROF_S16>, wave_kernel<10, SW, PROF_PAIR>, wave_kernel<10, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 11: {
      static const WaveFn t[2][3] = {
          {wave_kernel<11, SG, PROF_S16>, wave_kernel<11, SG, PROF_PAIR>, wave_kernel<11, SG, PROF_S32>},
          {wave_kernel<11, SW, PROF_S16>, wave_kernel<11, SW, PROF_PAIR>, wave_kernel<11, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 12: {
      static const WaveFn t[2][3] = {
          {wave_kernel<12, SG, PROF_S16>, wave_kernel<12, SG, PROF_PAIR>, wave_kernel<12, SG, PROF_S32>},
          {wave_kernel<12, SW, PROF_S16>, wave_kernel<12, SW, PROF_PAIR>, wave_kernel<12, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 13: {
      static const WaveFn t[2][3] = {
          {wave_kernel<13, SG, PROF_S16>, wave_kernel<13, SG, PROF_PAIR>, wave_kernel<13, SG, PROF_S32>},
          {wave_kernel<13, SW, PROF_S16>, wave_kernel<13, SW, PROF_PAIR>, wave_kernel<13, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 14: {
      static const WaveFn t[2][3] = {
          {wave_kernel<14, SG, PROF_S16>, wave_kernel<14, SG, PROF_PAIR>, wave_kernel<14, SG, PROF_S32>},
          {wave_kernel<14, SW, PROF_S16>, wave_kernel<14, SW, PROF_PAIR>, wave_kernel<14, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 15: {
      static const WaveFn t[2][3] = {
          {wave_kernel<15, SG, PROF_S16>, wave_kernel<15, SG, PROF_PAIR>, wave_kernel<15, SG, PROF_S32>},
          {wave_kernel<15, SW, PROF_S16>, wave_kernel<15, SW, PROF_PAIR>, wave_kernel<15, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 16: {
      static const WaveFn t[2][3] = {
          {wave_kernel<16, SG, PROF_S16>, wave_kernel<16, SG, PROF_PAIR>, wave_kernel<16, SG, PROF_S32>},
          {wave_kernel<16, SW, PROF_S16>, wave_kernel<16, SW, PROF_PAIR>, wave_kernel<16, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

BatchFn batch_fn_b(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 9: {
      static const BatchFn t[2][3] = {
          {batch_kernel<9, SG, PROF_S16>, batch_kernel<9, SG, PROF_PAIR>, batch_kernel<9, SG, PROF_S32>},
          {batch_kernel<9, SW, PROF_S16>, batch_kernel<9, SW, PROF_PAIR>, batch_kernel<9, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 10: {
      static const BatchFn t[2][3] = {
          {batch_kernel<10, SG, PROF_S16>, batch_kernel<10, SG, PROF_PAIR>, batch_kernel<10, SG, PROF_S32>},
          {batch_kernel<10, SW, PROF_S16>, batch_kernel<10, SW, PROF_PAIR>, batch_kernel<10, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 11: {
      static const BatchFn t[2][3] = {
          {batch_kernel<11, SG, PROF_S16>, batch_kernel<11, SG, PROF_PAIR>, batch_kernel<11, SG, PROF_S32>},
          {batch_kernel<11, SW, PROF_S16>, batch_kernel<11, SW, PROF_PAIR>, batch_kernel<11, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 12: {
      static const BatchFn t[2][3] = {
          {batch_kernel<12, SG, PROF_S16>, batch_kernel<12, SG, PROF_PAIR>, batch_kernel<12, SG, PROF_S32>},
          {batch_kernel<12, SW, PROF_S16>, batch_kernel<12, SW, PROF_PAIR>, batch_kernel<12, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 13: {
      static const BatchFn t[2][3] = {
          {batch_kernel<13, SG, PROF_S16>, batch_kernel<13, SG, PROF_PAIR>, batch_kernel<13, SG, PROF_S32>},
          {batch_kernel<13, SW, PROF_S16>, batch_kernel<13, SW, PROF_PAIR>, batch_kernel<13, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 14: {
      static const BatchFn t[2][3] = {
          {batch_kernel<14, SG, PROF_S16>, batch_kernel<14, SG, PROF_PAIR>, batch_kernel<14, SG, PROF_S32>},
          {batch_kernel<14, SW, PROF_S16>, batch_kernel<14, SW, PROF_PAIR>, batch_kernel<14, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 15: {
      static const BatchFn t[2][3] = {
          {batch_kernel<15, SG, PROF_S16>, batch_kernel<15, SG, PROF_PAIR>, batch_kernel<15, SG, PROF_S32>},
          {batch_kernel<15, SW, PROF_S16>, batch_kernel<15, SW, PROF_PAIR>, batch_kernel<15, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    case 16: {
      static const BatchFn t[2][3] = {
          {batch_kernel<16, SG, PROF_S16>, batch_kernel<16, SG, PROF_PAIR>, batch_kernel<16, SG, PROF_S32>},
          {batch_kernel<16, SW, PROF_S16>, batch_kernel<16, SW, PROF_PAIR>, batch_kernel<16, SW, PROF_S32>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

}  // namespace ish
