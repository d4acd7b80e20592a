// FP32 step and set-up kernels for transform lengths 8 .. 64.
#include "kernels_impl.cuh"

namespace af {
void fill_f32_3_6(KernelTable<float> &t) { fill_range<float, 3, 6>(t); }
}  // namespace af
