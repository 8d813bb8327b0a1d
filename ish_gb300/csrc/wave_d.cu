// wave_d.cu -- wavefront and batched kernels, K = 25..32.
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_d(int K, int mode, int layout) { return wave_table<0, 25, 26, 27, 28, 29, 30, 31, 32>(K, mode, layout); }
BatchFn batch_fn_d(int K, int mode, int layout) { return batch_table<0, 25, 26, 27, 28, 29, 30, 31, 32>(K, mode, layout); }

}  // namespace ish
