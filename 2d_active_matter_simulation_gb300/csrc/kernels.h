// Dispatch tables of the compiled step and set-up kernels, one per precision
// (FP32, FP64, double-float).  The tables are filled in kernels_f32.cu /
// kernels_f64.cu / kernels_df.cu, which instantiate the kernel templates for
// every supported power-of-two length.
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

// Coefficients of the integrating-factor table (k_lintab): wavenumber steps
// 2 pi / L, parameters in double, operator form (am_form).
struct LinCoef {
    double kxs, kys, dt, alpha, g0, g2;
    int form;
};

// Table entry {exp(L dt / 2), exp(L dt)} at half-plane index (kx, y): the
// wavenumbers, L(k) and both exponentials in double, each rounded to T once.
// L = -(1 - k^2)^2 - alpha (lin_func, ActFlow_V3-2.cu:1020-1033) or
// -alpha - g0 k^2 - g2 k^4.
template <typename T>
AF_HD cpx<T> lintab_value(const LinCoef &c, int ny, int kx, int y)
{
    const double kxd = c.kxs * kx, kyd = c.kys * (y < ny / 2 + 1 ? y : y - ny);
    const double k2 = kyd * kyd + kxd * kxd;
    const double L = c.form == 0 ? -(1 - k2) * (1 - k2) - c.alpha : -c.alpha - c.g0 * k2 - c.g2 * k2 * k2;
    return mk((T)exp(L * c.dt / 2), (T)exp(L * c.dt));
}

// CTAs of a step column-pass launch over ntp column tiles of W columns: the
// column groups, then one reducer CTA (ColPass::reduce_scalars).
inline int col_grid(const LaunchShape &s, int ntp, int W) { return (ntp * W + s.per_block - 1) / s.per_block + 1; }

// Column-pass launch shapes: 0 wide, 1 narrow, 2 wide radix 8 (FP32 only).
constexpr int NCOLV = 3;
// Row-pass launch shapes: 0 radix 8 in lockstep (RowPass), 1 in sequence with
// stashes (RowPassS; FP32 radix 16, double-float radix 8; Nx >= 512), 2 the
// lockstep pass with its input rows fetched by tensor-map copies (FP32,
// Nx >= 128; KernelTable::row_tma, used where a row's carried tiles fit one
// exchange buffer, else shape 0 runs).
constexpr int NROWV = 3;
constexpr int ROWV_TMA = 2;
constexpr int ROWS_LOG_MIN = 10;   // RowPassS needs Nx >= 512 (log2 9); it is built from 1024 up

template <typename T>
struct KernelTable {
    void (*row[LOG_MAX + 1][NROWV])(StepArgs<T>);   // [log2 Nx][shape]; null: shape not built
    LaunchShape row_shape[LOG_MAX + 1][NROWV];
    void (*col[LOG_MAX + 1][NCOLV][5])(StepArgs<T>);   // [log2 Ny][shape][mode]; null: shape not built
    LaunchShape col_shape[LOG_MAX + 1][NCOLV];
    void (*rowfwd[LOG_MAX + 1])(const T *, cpx<T> *, const cpx<T> *, int, int);
    LaunchShape rowfwd_shape[LOG_MAX + 1];
    void (*colfwd[LOG_MAX + 1])(const cpx<T> *, cpx<T> *, const cpx<T> *, int, int, int, int, int, int, int);
    LaunchShape colfwd_shape[LOG_MAX + 1];
    void (*row_tma[LOG_MAX + 1])(StepArgs<T>, RowTma);   // [log2 Nx]; null: not built
    LaunchShape row_tma_shape[LOG_MAX + 1];
    int row_tma_cap[LOG_MAX + 1];                          // complex values one staging buffer holds
    void (*tile)(const cpx<T> *, cpx<T> *, int, int, int, int, int *);   // [ny][nxh] -> tiled
    void (*untile)(const cpx<T> *, cpx<T> *, int, int, int);  // tiled -> [ny][nxh]
    void (*lintab)(cpx<T> *, int, int, int, LinCoef);         // integrating-factor table
};

const KernelTable<float> &kernels_f32();
const KernelTable<double> &kernels_f64();
const KernelTable<df> &kernels_df();

// In-place conversion of n reals between double and double-float (both 8
// bytes, so an array keeps its size and layout) on a CUDA stream; the state of
// an AM_DF64 simulation is exchanged with the host as double.
void df_from_double_async(void *data, size_t n, void *stream);
void df_to_double_async(void *data, size_t n, void *stream);

// Fillers of the tables, one per translation unit (ranges of log2 lengths).
void fill_f32_3_6(KernelTable<float> &t);
void fill_f32_7_8(KernelTable<float> &t);
void fill_f32_9(KernelTable<float> &t);
void fill_f32_10(KernelTable<float> &t);
void fill_f32_11(KernelTable<float> &t);
void fill_f32_12(KernelTable<float> &t);
void fill_f64_3_8(KernelTable<double> &t);
void fill_f64_9_10(KernelTable<double> &t);
void fill_f64_11(KernelTable<double> &t);
void fill_f64_12(KernelTable<double> &t);
void fill_df_3_5(KernelTable<df> &t);
void fill_df_6(KernelTable<df> &t);
void fill_df_7(KernelTable<df> &t);
void fill_df_8(KernelTable<df> &t);
void fill_df_9(KernelTable<df> &t);
void fill_df_10(KernelTable<df> &t);
void fill_df_11(KernelTable<df> &t);
void fill_df_12(KernelTable<df> &t);

// Batched forms of the step kernels: one launch covers every member of an
// ensemble (blockIdx.y = member), each member's arguments read from a device
// array.  FP32, grids 128..1024 per axis.
constexpr int BATCH_LOG_MIN = 7;
constexpr int BATCH_LOG_MAX = 10;

struct BatchTable {
    void (*row[LOG_MAX + 1][NROWV])(const StepArgs<float> *);       // [log2 Nx][shape]
    // the lockstep row pass with tensor-map row fetches over one map of every
    // simulation's fields (simulation i's field k is map field
    // args[i].tma_field0 + k); null: not built
    void (*row_tma[LOG_MAX + 1])(const StepArgs<float> *, RowTma);
    LaunchShape row_tma_shape[LOG_MAX + 1];
    int row_tma_cap[LOG_MAX + 1];   // complex values one staging buffer holds
    void (*col[LOG_MAX + 1][NCOLV][5])(const StepArgs<float> *);   // [log2 Ny][shape][mode]
};

// Column-pass launch shape (0 wide, 1 narrow, 2 wide radix 8) used for new
// simulations of this precision (am_precision) and log2 Ny: a process-wide
// table seeded with the measured rule (narrow below Ny = 2048) and updated by
// am_autotune / am_set_column_shape.
int col_variant(int prec, int logny);
void set_col_variant(int prec, int logny, int v);
bool col_variant_built(int prec, int logny, int v);
// Row-pass launch shape for new simulations of this precision and log2 Nx
// (0 lockstep, 1 in sequence with stashes), as col_variant.
int row_variant(int prec, int lognx);
void set_row_variant(int prec, int lognx, int v);
bool row_variant_built(int prec, int lognx, int v);

const BatchTable &kernels_batch_f32();

// A tensor map of FP32 tiled fields for the row pass's tensor-map fetch
// (actflow_api.cu): {8 floats of a tile row, Ny rows, nt column tiles,
// nfields fields field_stride bytes apart}, boxes of one row and `box` tiles.
bool encode_row_map(TmaDesc *out, void *base, int ny, int nt, int nfields, size_t field_stride, int box);

// Work-list kernels (kernels_queue.cu): one launch per pass over the runs of
// several size classes.  Item = the run's argument index, the CTA index within
// that run's own launch, log2 of the transform length (Nx for the row pass, Ny
// for the column pass), 128..1024.  Row pass with radix-8 passes, narrow
// column pass; CTAs of 128 threads.
struct WorkItem {
    int arg, block, log;
};
constexpr int QUEUE_LOG_MIN = 7;
constexpr int QUEUE_LOG_MAX = 10;
struct QueueTable {
    void (*row)(const StepArgs<float> *, const WorkItem *);
    void (*col[5])(const StepArgs<float> *, const WorkItem *);   // [mode], 1..4
    size_t row_smem, col_smem;
};
const QueueTable &kernels_queue_f32();
void fill_batch_7_8(BatchTable &t);
void fill_batch_9_10(BatchTable &t);

}  // namespace af
