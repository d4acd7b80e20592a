// Kernel entry points and dispatch-table construction.  The table of a
// precision is filled by several translation units, each instantiating a range
// of transform lengths (kernels_f32_*.cu, kernels_f64_*.cu, kernels_df_*.cu),
// so that they compile in parallel; kernels_f32.cu / kernels_f64.cu /
// kernels_df.cu assemble the tables.
#pragma once
#include "kernels.h"
#include "setup_kernels.cuh"

namespace af {

template <typename T, int LOG>
__global__ void __launch_bounds__(RowKernel<T, LOG>::THREADS, RowKernel<T, LOG>::MINB) k_row(StepArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    RowKernel<T, LOG>::body(a, threadIdx.x, blockIdx.x, smem, []() { __syncthreads(); });
}

template <typename T, int LOG>
__global__ void __launch_bounds__(RowKernel<T, LOG>::THREADS, RowKernel<T, LOG>::MINB)
    k_row_tma(StepArgs<T> a, const __grid_constant__ RowTma m)
{
    extern __shared__ __align__(16) unsigned char smem[];
    RowKernel<T, LOG>::body(a, threadIdx.x, blockIdx.x, smem, []() { __syncthreads(); }, &m);
}

template <typename T, int LOG>
__global__ void __launch_bounds__(RowPassS<T, LOG>::THREADS, RowPassS<T, LOG>::MINB) k_rows(StepArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    RowPassS<T, LOG>::body(a, threadIdx.x, blockIdx.x, smem, []() { __syncthreads(); });
}

template <typename T, int LOG, int MODE, int VAR>
__global__ void __launch_bounds__(ColPass<T, LOG, MODE, VAR>::THREADS, ColPass<T, LOG, MODE, VAR>::MINB)
    k_col(StepArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    ColPass<T, LOG, MODE, VAR>::body(a, threadIdx.x, blockIdx.x, smem, []() { __syncthreads(); });
}

template <typename T, int LOG>
__global__ void __launch_bounds__(RowFwd<T, LOG>::THREADS)
    k_rowfwd(const T *src, cpx<T> *dst, const cpx<T> *twx, int ny, int nt)
{
    extern __shared__ __align__(16) unsigned char smem[];
    RowFwd<T, LOG>::body(src, dst, twx, ny, nt, threadIdx.x, blockIdx.x, smem, []() { __syncthreads(); });
}

template <typename T, int LOG>
__global__ void __launch_bounds__(ColFwd<T, LOG>::THREADS)
    k_colfwd(const cpx<T> *src, cpx<T> *dst, const cpx<T> *twy, int nx, int ny, int nxh, int nt, int apply_mask,
             int dealias, int rsq)
{
    extern __shared__ __align__(16) unsigned char smem[];
    ColFwd<T, LOG>::body(src, dst, twy, nx, ny, nxh, nt, apply_mask, dealias, rsq, threadIdx.x, blockIdx.x, smem,
                         []() { __syncthreads(); });
}

// Reference half-plane layout [ny][nxh] <-> tiled layout; padding columns
// zero.  With `outside` non-null, sets *outside = 1 if the state has a nonzero
// value at a mode the 1/2 rule removes (the device form of
// state_inside_half_mask; every writer stores the same value).
template <typename T>
__global__ void k_tile(const cpx<T> *src, cpx<T> *dst, int ny, int nxh, int nt, int nx, int *outside)
{
    constexpr int W = Tile<T>::W;
    size_t total = (size_t)nt * W * ny;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        int c = (int)(i % W);
        size_t rest = i / W;
        int y = (int)(rest % ny);
        int t = (int)(rest / ny);
        int kx = t * W + c;
        const cpx<T> v = kx < nxh ? src[(size_t)y * nxh + kx] : mk<T>(0, 0);
        dst[i] = v;
        if (outside && (v.x != T(0) || v.y != T(0)) && !mask_at(1, 0, nx, ny, kx, y)) *outside = 1;
    }
}

template <typename T>
__global__ void k_untile(const cpx<T> *src, cpx<T> *dst, int ny, int nxh, int nt)
{
    size_t total = (size_t)ny * nxh;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        int y = (int)(i / nxh), kx = (int)(i % nxh);
        dst[i] = src[tidx<T>(kx, y, ny)];
    }
}

// Integrating factors {exp(L dt / 2), exp(L dt)} at every half-plane (kx, ky)
// (lintab_value), tiled like the fields; padding columns zero.
template <typename T>
__global__ void k_lintab(cpx<T> *tab, int nx, int ny, int nt, LinCoef c)
{
    constexpr int W = Tile<T>::W;
    const int nxh = nx / 2 + 1;
    const size_t total = (size_t)nt * W * ny;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int cc = (int)(i % W);
        const size_t rest = i / W;
        const int y = (int)(rest % ny);
        const int kx = (int)(rest / ny) * W + cc;
        tab[i] = kx < nxh ? lintab_value<T>(c, ny, kx, y) : mk<T>(0, 0);
    }
}

template <typename T, int LOG, int HI>
struct Fill {
    template <int V>
    static void fill_col(KernelTable<T> &t)
    {
        t.col[LOG][V][0] = k_col<T, LOG, 0, V>;
        t.col[LOG][V][1] = k_col<T, LOG, 1, V>;
        t.col[LOG][V][2] = k_col<T, LOG, 2, V>;
        t.col[LOG][V][3] = k_col<T, LOG, 3, V>;
        t.col[LOG][V][4] = k_col<T, LOG, 4, V>;
        using CP = ColPass<T, LOG, 1, V>;
        t.col_shape[LOG][V] = {CP::THREADS, CP::smem_bytes(), CP::COLS};
    }
    static void run(KernelTable<T> &t)
    {
        t.row[LOG][0] = k_row<T, LOG>;
        t.row_shape[LOG][0] = {RowKernel<T, LOG>::THREADS, RowKernel<T, LOG>::smem_bytes(), RowKernel<T, LOG>::ROWS};
        // row shape 1, transforms in sequence: FP32 (radix 16) and
        // double-float (radix 8), Nx >= 1024
        if constexpr (std::is_same_v<T, float> && !RowKernel<T, LOG>::SINGLE && LOG >= 7) {
            // row shape 2: the lockstep pass with tensor-map row fetches
            using RK = RowKernel<T, LOG>;
            t.row_tma[LOG] = k_row_tma<T, LOG>;
            t.row_tma_shape[LOG] = {RK::THREADS, RK::smem_bytes_tma(), RK::ROWS};
            t.row_tma_cap[LOG] = RK::BUFS;
        }
        if constexpr ((sizeof(T) == 4 || std::is_same_v<T, df>) && LOG >= ROWS_LOG_MIN) {
            t.row[LOG][1] = k_rows<T, LOG>;
            t.row_shape[LOG][1] = {RowPassS<T, LOG>::THREADS, RowPassS<T, LOG>::smem_bytes(), RowPassS<T, LOG>::ROWS};
        }
        if constexpr (std::is_same_v<T, df>) {
            // double-float: the default shape of the length only (each
            // instantiation of these long unrolled kernels costs compile time)
            fill_col<(LOG < 11 ? 1 : 0)>(t);
        } else {
            fill_col<0>(t);
            fill_col<1>(t);
        }
        if constexpr (sizeof(T) == 4) fill_col<2>(t);   // wide radix 8: FP32 only
        t.rowfwd[LOG] = k_rowfwd<T, LOG>;
        t.rowfwd_shape[LOG] = {RowFwd<T, LOG>::THREADS, RowFwd<T, LOG>::smem_bytes(), RowFwd<T, LOG>::ROWS};
        t.colfwd[LOG] = k_colfwd<T, LOG>;
        t.colfwd_shape[LOG] = {ColFwd<T, LOG>::THREADS, ColFwd<T, LOG>::smem_bytes(), ColFwd<T, LOG>::TILES};
        if constexpr (LOG < HI) Fill<T, LOG + 1, HI>::run(t);
    }
};

// Entries for log2 lengths LO..HI.
template <typename T, int LO, int HI>
void fill_range(KernelTable<T> &t)
{
    Fill<T, LO, HI>::run(t);
}

// The layout-conversion kernels.
template <typename T>
void fill_common(KernelTable<T> &t)
{
    t.tile = k_tile<T>;
    t.untile = k_untile<T>;
    t.lintab = k_lintab<T>;
}

}  // namespace af
