// FP64 step and set-up kernels for transform lengths 4096.
#include "kernels_impl.cuh"

namespace af {
void fill_f64_12(KernelTable<double> &t) { fill_range<double, 12, 12>(t); }
}  // namespace af
