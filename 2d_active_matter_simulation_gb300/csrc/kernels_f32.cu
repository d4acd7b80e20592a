// FP32 instantiations of the step and set-up kernels (Nx, Ny = 8 .. 4096).
#include "kernels_impl.cuh"

namespace af {
const KernelTable<float> &kernels_f32()
{
    static const KernelTable<float> t = make_table<float>();
    return t;
}
}  // namespace af
