// wave_f.cu -- wavefront and batched kernels, even K = 50..64.
#include "kernels.cuh"
#include "wave.cuh"

namespace ish {

WaveFn wave_fn_f(int K, int mode, int layout) { return wave_table<0, 50, 52, 54, 56, 58, 60, 62, 64>(K, mode, layout); }
BatchFn batch_fn_f(int K, int mode, int layout) { return batch_table<0, 50, 52, 54, 56, 58, 60, 62, 64>(K, mode, layout); }

}  // namespace ish
