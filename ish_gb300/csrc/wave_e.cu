// wave_e.cu -- wavefront and batched kernels, even K = 34..48.
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_e(int K, int mode, int layout) { return wave_table<0, 34, 36, 38, 40, 42, 44, 46, 48>(K, mode, layout); }
BatchFn batch_fn_e(int K, int mode, int layout) { return batch_table<0, 34, 36, 38, 40, 42, 44, 46, 48>(K, mode, layout); }

}  // namespace ish
