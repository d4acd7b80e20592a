// FP32 step and set-up kernels for transform lengths 2048.
#include "kernels_impl.cuh"

namespace af {
void fill_f32_11(KernelTable<float> &t) { fill_range<float, 11, 11>(t); }
}  // namespace af
