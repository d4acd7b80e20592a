// FP64 kernel table (Nx, Ny = 8 .. 4096), assembled from the units that
// instantiate each range of lengths (kernels_f64_*.cu).
#include "kernels_impl.cuh"

namespace af {
const KernelTable<double> &kernels_f64()
{
    static const KernelTable<double> t = []() {
        KernelTable<double> k{};
        fill_f64_3_8(k);
        fill_f64_9_10(k);
        fill_f64_11(k);
        fill_f64_12(k);
        fill_common<double>(k);
        return k;
    }();
    return t;
}
}  // namespace af
