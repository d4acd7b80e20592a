// FP64 instantiations of the step and set-up kernels (Nx, Ny = 8 .. 4096).
#include "kernels_impl.cuh"

namespace af {
const KernelTable<double> &kernels_f64()
{
    static const KernelTable<double> t = make_table<double>();
    return t;
}
}  // namespace af
