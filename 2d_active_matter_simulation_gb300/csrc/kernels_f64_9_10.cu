// FP64 step and set-up kernels for transform lengths 512 .. 1024.
#include "kernels_impl.cuh"

namespace af {
void fill_f64_9_10(KernelTable<double> &t) { fill_range<double, 9, 10>(t); }
}  // namespace af
