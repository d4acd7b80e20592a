// FP32 kernel table (Nx, Ny = 8 .. 4096), assembled from the units that
// instantiate each range of lengths (kernels_f32_*.cu).
#include "kernels_impl.cuh"

namespace af {
const KernelTable<float> &kernels_f32()
{
    static const KernelTable<float> t = []() {
        KernelTable<float> k{};
        fill_f32_3_6(k);
        fill_f32_7_8(k);
        fill_f32_9(k);
        fill_f32_10(k);
        fill_f32_11(k);
        fill_f32_12(k);
        fill_common<float>(k);
        return k;
    }();
    return t;
}
}  // namespace af
