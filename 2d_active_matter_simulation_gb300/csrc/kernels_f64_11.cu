// FP64 step and set-up kernels for transform lengths 2048.
#include "kernels_impl.cuh"

namespace af {
void fill_f64_11(KernelTable<double> &t) { fill_range<double, 11, 11>(t); }
}  // namespace af
