// FP64 step and set-up kernels for transform lengths 8 .. 256.
#include "kernels_impl.cuh"

namespace af {
void fill_f64_3_8(KernelTable<double> &t) { fill_range<double, 3, 8>(t); }
}  // namespace af
