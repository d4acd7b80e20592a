// Batched FP32 step kernels (blockIdx.y = ensemble member), grids 128..1024;
// instantiated by kernels_batch.cu (128, 256) and kernels_batch_9_10.cu
// (512, 1024), which compile in parallel.
#pragma once
#include "kernels_impl.cuh"

namespace af {

template <typename T, int LOG>
__global__ void __launch_bounds__(RowKernel<T, LOG>::THREADS, RowKernel<T, LOG>::MINB)
    k_row_b(const StepArgs<T> *__restrict__ args)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const StepArgs<T> a = args[blockIdx.y];
    RowKernel<T, LOG>::body(a, threadIdx.x, blockIdx.x, smem, []() { __syncthreads(); });
}

template <typename T, int LOG>
__global__ void __launch_bounds__(RowKernel<T, LOG>::THREADS, RowKernel<T, LOG>::MINB)
    k_row_b_tma(const StepArgs<T> *__restrict__ args, const __grid_constant__ RowTma m)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const StepArgs<T> a = args[blockIdx.y];
    RowKernel<T, LOG>::body(a, threadIdx.x, blockIdx.x, smem, []() { __syncthreads(); }, &m, a.tma_field0);
}

template <typename T, int LOG>
__global__ void __launch_bounds__(RowPassS<T, LOG>::THREADS, RowPassS<T, LOG>::MINB)
    k_rows_b(const StepArgs<T> *__restrict__ args)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const StepArgs<T> a = args[blockIdx.y];
    RowPassS<T, LOG>::body(a, threadIdx.x, blockIdx.x, smem, []() { __syncthreads(); });
}

template <typename T, int LOG, int MODE, int VAR>
__global__ void __launch_bounds__(ColPass<T, LOG, MODE, VAR>::THREADS, ColPass<T, LOG, MODE, VAR>::MINB)
    k_col_b(const StepArgs<T> *__restrict__ args)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const StepArgs<T> a = args[blockIdx.y];
    ColPass<T, LOG, MODE, VAR>::body(a, threadIdx.x, blockIdx.x, smem, []() { __syncthreads(); });
}

template <int LOG, int HI>
struct FillB {
    static void run(BatchTable &t)
    {
        t.row[LOG][0] = k_row_b<float, LOG>;
        if constexpr (!RowKernel<float, LOG>::SINGLE) {
            using RK = RowKernel<float, LOG>;
            t.row_tma[LOG] = k_row_b_tma<float, LOG>;
            t.row_tma_shape[LOG] = {RK::THREADS, RK::smem_bytes_tma(), RK::ROWS};
            t.row_tma_cap[LOG] = RK::BUFS;
        }
        if constexpr (LOG >= ROWS_LOG_MIN) t.row[LOG][1] = k_rows_b<float, LOG>;
        t.col[LOG][0][0] = k_col_b<float, LOG, 0, 0>;
        t.col[LOG][0][1] = k_col_b<float, LOG, 1, 0>;
        t.col[LOG][0][2] = k_col_b<float, LOG, 2, 0>;
        t.col[LOG][0][3] = k_col_b<float, LOG, 3, 0>;
        t.col[LOG][0][4] = k_col_b<float, LOG, 4, 0>;
        t.col[LOG][1][0] = k_col_b<float, LOG, 0, 1>;
        t.col[LOG][1][1] = k_col_b<float, LOG, 1, 1>;
        t.col[LOG][1][2] = k_col_b<float, LOG, 2, 1>;
        t.col[LOG][1][3] = k_col_b<float, LOG, 3, 1>;
        t.col[LOG][1][4] = k_col_b<float, LOG, 4, 1>;
        t.col[LOG][2][0] = k_col_b<float, LOG, 0, 2>;
        t.col[LOG][2][1] = k_col_b<float, LOG, 1, 2>;
        t.col[LOG][2][2] = k_col_b<float, LOG, 2, 2>;
        t.col[LOG][2][3] = k_col_b<float, LOG, 3, 2>;
        t.col[LOG][2][4] = k_col_b<float, LOG, 4, 2>;
        if constexpr (LOG < HI) FillB<LOG + 1, HI>::run(t);
    }
};


}  // namespace af
