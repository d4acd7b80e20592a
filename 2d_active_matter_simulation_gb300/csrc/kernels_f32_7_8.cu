// FP32 step and set-up kernels for transform lengths 128 .. 256.
#include "kernels_impl.cuh"

namespace af {
void fill_f32_7_8(KernelTable<float> &t) { fill_range<float, 7, 8>(t); }
}  // namespace af
