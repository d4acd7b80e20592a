// FP32 step and set-up kernels for transform lengths 4096.
#include "kernels_impl.cuh"

namespace af {
void fill_f32_12(KernelTable<float> &t) { fill_range<float, 12, 12>(t); }
}  // namespace af
