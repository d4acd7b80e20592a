// Double-float kernel table (Nx, Ny = 8 .. 4096), assembled from the units
// that instantiate each range of lengths (kernels_df_*.cu), and the
// conversions between double and double-float.
#include <cuda_runtime.h>

#include "kernels_impl.cuh"

namespace af {

const KernelTable<df> &kernels_df()
{
    static const KernelTable<df> t = []() {
        KernelTable<df> k{};
        fill_df_3_5(k);
        fill_df_6(k);
        fill_df_7(k);
        fill_df_8(k);
        fill_df_9(k);
        fill_df_10(k);
        fill_df_11(k);
        fill_df_12(k);
        fill_common<df>(k);
        return k;
    }();
    return t;
}

namespace {
// Each thread converts whole elements in place: the 8 bytes of element i are
// read, then written, by the same thread.
__global__ void k_df_from_double(void *data, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double d = static_cast<const double *>(data)[i];
        static_cast<df *>(data)[i] = df(d);
    }
}
__global__ void k_df_to_double(void *data, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const df v = static_cast<const df *>(data)[i];
        static_cast<double *>(data)[i] = (double)v;
    }
}
}  // namespace

void df_from_double_async(void *data, size_t n, void *stream)
{
    k_df_from_double<<<1024, 256, 0, (cudaStream_t)stream>>>(data, n);
}
void df_to_double_async(void *data, size_t n, void *stream)
{
    k_df_to_double<<<1024, 256, 0, (cudaStream_t)stream>>>(data, n);
}

}  // namespace af
