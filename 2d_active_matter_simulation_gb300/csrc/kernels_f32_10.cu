// FP32 step and set-up kernels for transform lengths 1024.
#include "kernels_impl.cuh"

namespace af {
void fill_f32_10(KernelTable<float> &t) { fill_range<float, 10, 10>(t); }
}  // namespace af
