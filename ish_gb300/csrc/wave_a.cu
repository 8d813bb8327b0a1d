// wave_a.cu -- wavefront and batched kernels, K = 1..8.
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_a(int K, int mode, int layout) { return wave_table<0, 1, 2, 3, 4, 5, 6, 7, 8>(K, mode, layout); }
BatchFn batch_fn_a(int K, int mode, int layout) { return batch_table<0, 1, 2, 3, 4, 5, 6, 7, 8>(K, mode, layout); }

}  // namespace ish
