// FP32 step and set-up kernels for transform lengths 512.
#include "kernels_impl.cuh"

namespace af {
void fill_f32_9(KernelTable<float> &t) { fill_range<float, 9, 9>(t); }
}  // namespace af
