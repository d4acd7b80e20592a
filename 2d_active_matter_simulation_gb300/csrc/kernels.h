// Dispatch tables of the compiled step and set-up kernels, one per precision.
// The tables are filled in kernels_f32.cu / kernels_f64.cu, which instantiate
// the kernel templates for every supported power-of-two length.
#pragma once
#include <cstddef>

#include "step_kernels.cuh"

namespace af {

constexpr int LOG_MIN = 3;    // 8
constexpr int LOG_MAX = 12;   // 4096

struct LaunchShape {
    int threads = 0;
    size_t smem = 0;
    int per_block = 0;        // rows (row kernels), columns (step column kernels) or column
                              // tiles (set-up column kernels) per CTA
};

// CTAs of a step column-pass launch over ntp column tiles of W columns.
inline int col_grid(const LaunchShape &s, int ntp, int W) { return (ntp * W + s.per_block - 1) / s.per_block; }

template <typename T>
struct KernelTable {
    void (*row[LOG_MAX + 1])(StepArgs<T>);
    LaunchShape row_shape[LOG_MAX + 1];
    void (*col[LOG_MAX + 1][5])(StepArgs<T>);   // [log2 Ny][mode]
    LaunchShape col_shape[LOG_MAX + 1];
    void (*rowfwd[LOG_MAX + 1])(const T *, cpx<T> *, const cpx<T> *, int, int);
    LaunchShape rowfwd_shape[LOG_MAX + 1];
    void (*colfwd[LOG_MAX + 1])(const cpx<T> *, cpx<T> *, const cpx<T> *, int, int, int, int, int, int, int);
    LaunchShape colfwd_shape[LOG_MAX + 1];
    void (*tile)(const cpx<T> *, cpx<T> *, int, int, int);    // [ny][nxh] -> tiled
    void (*untile)(const cpx<T> *, cpx<T> *, int, int, int);  // tiled -> [ny][nxh]
};

const KernelTable<float> &kernels_f32();
const KernelTable<double> &kernels_f64();

// Batched forms of the step kernels: one launch covers every member of an
// ensemble (blockIdx.y = member), each member's arguments read from a device
// array.  FP32, grids 128..1024 per axis.
constexpr int BATCH_LOG_MIN = 7;
constexpr int BATCH_LOG_MAX = 10;

struct BatchTable {
    void (*row[LOG_MAX + 1])(const StepArgs<float> *);
    void (*col[LOG_MAX + 1][5])(const StepArgs<float> *);
};

const BatchTable &kernels_batch_f32();

}  // namespace af
