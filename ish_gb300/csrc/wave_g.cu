// wave_g.cu -- register-lean builds (128 threads x 2 blocks), even K = 34..48.
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_g(int K, int mode, int layout) { return wave_table<1, 34, 36, 38, 40, 42, 44, 46, 48>(K, mode, layout); }
BatchFn batch_fn_g(int K, int mode, int layout) { return batch_table<1, 34, 36, 38, 40, 42, 44, 46, 48>(K, mode, layout); }

}  // namespace ish
