// wave_c.cu -- wavefront and batched kernels, K = 17..24.
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_c(int K, int mode, int layout) { return wave_table<0, 17, 18, 19, 20, 21, 22, 23, 24>(K, mode, layout); }
BatchFn batch_fn_c(int K, int mode, int layout) { return batch_table<0, 17, 18, 19, 20, 21, 22, 23, 24>(K, mode, layout); }

}  // namespace ish
