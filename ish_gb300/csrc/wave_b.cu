// wave_b.cu -- wavefront and batched kernels, K = 9..16.
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_b(int K, int mode, int layout) { return wave_table<0, 9, 10, 11, 12, 13, 14, 15, 16>(K, mode, layout); }
BatchFn batch_fn_b(int K, int mode, int layout) { return batch_table<0, 9, 10, 11, 12, 13, 14, 15, 16>(K, mode, layout); }

}  // namespace ish
