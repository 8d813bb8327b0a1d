// wave_h.cu -- register-lean (128 x 3) wavefront kernel instantiations for K = 25, 26, 27, 28, 29, 30, 31, 32
// (see wave_threads_lean / wave_blocks_lean in kernels.cuh).
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_h(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 25: {
      static const WaveFn t[2][3] = {
          {wave_kernel<25, SG, PROF_S16, 1>, wave_kernel<25, SG, PROF_PAIR, 1>, wave_kernel<25, SG, PROF_S32, 1>},
          {wave_kernel<25, SW, PROF_S16, 1>, wave_kernel<25, SW, PROF_PAIR, 1>, wave_kernel<25, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 26: {
      static const WaveFn t[2][3] = {
          {wave_kernel<26, SG, PROF_S16, 1>, wave_kernel<26, SG, PROF_PAIR, 1>, wave_kernel<26, SG, PROF_S32, 1>},
          {wave_kernel<26, SW, PROF_S16, 1>, wave_kernel<26, SW, PROF_PAIR, 1>, wave_kernel<26, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 27: {
      static const WaveFn t[2][3] = {
          {wave_kernel<27, SG, PROF_S16, 1>, wave_kernel<27, SG, PROF_PAIR, 1>, wave_kernel<27, SG, PROF_S32, 1>},
          {wave_kernel<27, SW, PROF_S16, 1>, wave_kernel<27, SW, PROF_PAIR, 1>, wave_kernel<27, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 28: {
      static const WaveFn t[2][3] = {
          {wave_kernel<28, SG, PROF_S16, 1>, wave_kernel<28, SG, PROF_PAIR, 1>, wave_kernel<28, SG, PROF_S32, 1>},
          {wave_kernel<28, SW, PROF_S16, 1>, wave_kernel<28, SW, PROF_PAIR, 1>, wave_kernel<28, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 29: {
      static const WaveFn t[2][3] = {
          {wave_kernel<29, SG, PROF_S16, 1>, wave_kernel<29, SG, PROF_PAIR, 1>, wave_kernel<29, SG, PROF_S32, 1>},
          {wave_kernel<29, SW, PROF_S16, 1>, wave_kernel<29, SW, PROF_PAIR, 1>, wave_kernel<29, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 30: {
      static const WaveFn t[2][3] = {
          {wave_kernel<30, SG, PROF_S16, 1>, wave_kernel<30, SG, PROF_PAIR, 1>, wave_kernel<30, SG, PROF_S32, 1>},
          {wave_kernel<30, SW, PROF_S16, 1>, wave_kernel<30, SW, PROF_PAIR, 1>, wave_kernel<30, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 31: {
      static const WaveFn t[2][3] = {
          {wave_kernel<31, SG, PROF_S16, 1>, wave_kernel<31, SG, PROF_PAIR, 1>, wave_kernel<31, SG, PROF_S32, 1>},
          {wave_kernel<31, SW, PROF_S16, 1>, wave_kernel<31, SW, PROF_PAIR, 1>, wave_kernel<31, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 32: {
      static const WaveFn t[2][3] = {
          {wave_kernel<32, SG, PROF_S16, 1>, wave_kernel<32, SG, PROF_PAIR, 1>, wave_kernel<32, SG, PROF_S32, 1>},
          {wave_kernel<32, SW, PROF_S16, 1>, wave_kernel<32, SW, PROF_PAIR, 1>, wave_kernel<32, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

BatchFn batch_fn_h(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  switch (K) {
    case 25: {
      static const BatchFn t[2][3] = {
          {batch_kernel<25, SG, PROF_S16, 1>, batch_kernel<25, SG, PROF_PAIR, 1>, batch_kernel<25, SG, PROF_S32, 1>},
          {batch_kernel<25, SW, PROF_S16, 1>, batch_kernel<25, SW, PROF_PAIR, 1>, batch_kernel<25, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 26: {
      static const BatchFn t[2][3] = {
          {batch_kernel<26, SG, PROF_S16, 1>, batch_kernel<26, SG, PROF_PAIR, 1>, batch_kernel<26, SG, PROF_S32, 1>},
          {batch_kernel<26, SW, PROF_S16, 1>, batch_kernel<26, SW, PROF_PAIR, 1>, batch_kernel<26, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 27: {
      static const BatchFn t[2][3] = {
          {batch_kernel<27, SG, PROF_S16, 1>, batch_kernel<27, SG, PROF_PAIR, 1>, batch_kernel<27, SG, PROF_S32, 1>},
          {batch_kernel<27, SW, PROF_S16, 1>, batch_kernel<27, SW, PROF_PAIR, 1>, batch_kernel<27, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 28: {
      static const BatchFn t[2][3] = {
          {batch_kernel<28, SG, PROF_S16, 1>, batch_kernel<28, SG, PROF_PAIR, 1>, batch_kernel<28, SG, PROF_S32, 1>},
          {batch_kernel<28, SW, PROF_S16, 1>, batch_kernel<28, SW, PROF_PAIR, 1>, batch_kernel<28, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 29: {
      static const BatchFn t[2][3] = {
          {batch_kernel<29, SG, PROF_S16, 1>, batch_kernel<29, SG, PROF_PAIR, 1>, batch_kernel<29, SG, PROF_S32, 1>},
          {batch_kernel<29, SW, PROF_S16, 1>, batch_kernel<29, SW, PROF_PAIR, 1>, batch_kernel<29, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 30: {
      static const BatchFn t[2][3] = {
          {batch_kernel<30, SG, PROF_S16, 1>, batch_kernel<30, SG, PROF_PAIR, 1>, batch_kernel<30, SG, PROF_S32, 1>},
          {batch_kernel<30, SW, PROF_S16, 1>, batch_kernel<30, SW, PROF_PAIR, 1>, batch_kernel<30, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 31: {
      static const BatchFn t[2][3] = {
          {batch_kernel<31, SG, PROF_S16, 1>, batch_kernel<31, SG, PROF_PAIR, 1>, batch_kernel<31, SG, PROF_S32, 1>},
          {batch_kernel<31, SW, PROF_S16, 1>, batch_kernel<31, SW, PROF_PAIR, 1>, batch_kernel<31, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    case 32: {
      static const BatchFn t[2][3] = {
          {batch_kernel<32, SG, PROF_S16, 1>, batch_kernel<32, SG, PROF_PAIR, 1>, batch_kernel<32, SG, PROF_S32, 1>},
          {batch_kernel<32, SW, PROF_S16, 1>, batch_kernel<32, SW, PROF_PAIR, 1>, batch_kernel<32, SW, PROF_S32, 1>}};
      return t[mode == SW][layout];
    }
    default:
      return nullptr;
  }
}

}  // namespace ish
