// C ABI of the actflow solver (declared in include/actflow.h).
//
// One handle = one simulation on one GPU stream.  Device memory per handle
// (complex half-plane fields in the tiled layout, s = sizeof(cpx<T>)):
//   u0, acc            spectral state w_old / w_new                2 fields
//   fa, fx, fy         next stage input a, ux, uy in (kx, y)        3 fields
//   P, Q               real-space products after R2C along x        2 fields
//   stage              host <-> device staging in the reference layout
// plus per-row sums, scalars, the energy ring and small tables.  A step is 8
// kernel launches (row pass + column pass per RK stage), captured once into a
// CUDA graph and replayed.
#include <cuda.h>   // CUtensorMap and its encoder's types (the encoder is reached through the runtime)
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <random>
#include <string>
#include <type_traits>
#include <vector>

#include "actflow.h"
#include "handle_internal.h"
#include "host_tables.h"
#include "kernels.h"

using namespace af;

namespace {

constexpr int ECAP = 4096;   // energy ring entries per handle

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
int ilog2(int n)
{
    int l = 0;
    while ((1 << l) < n) l++;
    return l;
}

}  // namespace

struct am_handle {
    am_params p{};
    int nxh = 0, nt = 0, W = 0, lognx = 0, logny = 0;
    int colv = 0;                  // column-pass launch shape (0 wide, 1 narrow, 2 wide radix 8)
    int rowv = 0;                  // row-pass launch shape (0 radix 8, 1 radix 16 with stashes)
    int prec = AM_FP32;            // am_precision
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int device = 0;
    // device memory
    void *u0 = nullptr, *acc = nullptr, *fa = nullptr, *fx = nullptr, *fy = nullptr, *P = nullptr, *Q = nullptr;
    void *stage = nullptr, *twx = nullptr, *twy = nullptr, *kxt = nullptr, *kyt = nullptr;
    void *lin = nullptr;           // integrating-factor table (AM_IF_DOUBLE), one field
    double *rowp = nullptr, *energy = nullptr;
    Scalars *sc = nullptr;
    long long bytes = 0;
    // graph of one step; graph of the step's four row passes alone (measurement)
    cudaGraphExec_t graph = nullptr, graph_rows = nullptr;
    bool state_loaded = false;
    std::string err;
    // kernel arguments (scalar part filled at create)
    StepArgs<float> a32{};
    StepArgs<double> a64{};
    StepArgs<df> adf{};
    // row shape 2 (FP32): tensor maps of the row pass's inputs for the current
    // pruning, and whether a row's carried tiles fit its staging buffer
    RowTma tma{};
    bool tma_ok = false;
};

// Calls f with a value of the state type of precision prec: float (AM_FP32),
// double (AM_FP64) or double-float (AM_DF64).
template <class F>
static am_status with_type(int prec, F &&f)
{
    if (prec == AM_FP64) return f(double{});
    if (prec == AM_DF64) return f(df{});
    return f(float{});
}

// Host-side element type of a state of type T: double-float states are
// exchanged with the host as double.
template <typename T>
using HostT = std::conditional_t<std::is_same_v<T, df>, double, T>;

static am_status cuda_fail(am_handle *h, cudaError_t e, const char *what)
{
    if (h) {
        h->err = std::string(what) + ": " + cudaGetErrorString(e);
    }
    return e == cudaErrorMemoryAllocation ? AM_ERR_OOM : AM_ERR_CUDA;
}

#define CK(h, call)                                            \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
    } while (0)

template <typename T>
static StepArgs<T> &args_of(am_handle *h);
template <>
StepArgs<float> &args_of<float>(am_handle *h) { return h->a32; }
template <>
StepArgs<double> &args_of<double>(am_handle *h) { return h->a64; }
template <>
StepArgs<df> &args_of<df>(am_handle *h) { return h->adf; }

template <typename T>
static const KernelTable<T> &table();
template <>
const KernelTable<float> &table<float>() { return kernels_f32(); }
template <>
const KernelTable<double> &table<double>() { return kernels_f64(); }
template <>
const KernelTable<df> &table<df>() { return kernels_df(); }

template <typename T>
static am_status alloc_and_tables(am_handle *h)
{
    const am_params &p = h->p;
    const int nx = p.nx, ny = p.ny;
    const int W = Tile<T>::W;
    h->W = W;
    h->nxh = nx / 2 + 1;
    h->nt = (h->nxh + W - 1) / W;
    const size_t field = (size_t)h->nt * W * ny * sizeof(cpx<T>);
    const size_t stage = (size_t)ny * h->nxh * sizeof(cpx<T>);
    void **fields[] = {&h->u0, &h->acc, &h->fa, &h->fx, &h->fy, &h->P, &h->Q};
    for (void **f : fields) {
        CK(h, cudaMallocAsync(f, field, h->stream));
        CK(h, cudaMemsetAsync(*f, 0, field, h->stream));
        h->bytes += field;
    }
    CK(h, cudaMallocAsync(&h->stage, stage, h->stream));
    h->bytes += stage;
    if (use_if_table(p)) {
        CK(h, cudaMallocAsync(&h->lin, field, h->stream));
        h->bytes += field;
    }
    CK(h, cudaMallocAsync(&h->twx, nx * sizeof(cpx<T>), h->stream));
    CK(h, cudaMallocAsync(&h->twy, ny * sizeof(cpx<T>), h->stream));
    CK(h, cudaMallocAsync(&h->kxt, h->nt * W * sizeof(T), h->stream));
    CK(h, cudaMallocAsync(&h->kyt, ny * sizeof(T), h->stream));
    CK(h, cudaMallocAsync(&h->rowp, side_bytes(ny), h->stream));
    CK(h, cudaMemsetAsync(h->rowp, 0, side_bytes(ny), h->stream));
    CK(h, cudaMallocAsync(&h->energy, ECAP * sizeof(double), h->stream));
    CK(h, cudaMallocAsync(&h->sc, sizeof(Scalars), h->stream));
    h->bytes += nx * sizeof(cpx<T>) + ny * sizeof(cpx<T>) + h->nt * W * sizeof(T) + ny * sizeof(T) +
                side_bytes(ny) + ECAP * sizeof(double) + sizeof(Scalars);

    HostTables<T> t;
    StepArgs<T> &a = args_of<T>(h);
    host_setup<T>(p, t, a, ECAP);
    CK(h, cudaMemcpyAsync(h->twx, t.twx.data(), nx * sizeof(cpx<T>), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->twy, t.twy.data(), ny * sizeof(cpx<T>), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->kxt, t.kx.data(), t.kx.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->kyt, t.ky.data(), t.ky.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    a.u0 = (cpx<T> *)h->u0;
    a.acc = (cpx<T> *)h->acc;
    a.fa = (cpx<T> *)h->fa;
    a.fx = (cpx<T> *)h->fx;
    a.fy = (cpx<T> *)h->fy;
    a.P = (cpx<T> *)h->P;
    a.Q = (cpx<T> *)h->Q;
    a.twx = (const cpx<T> *)h->twx;
    a.twy = (const cpx<T> *)h->twy;
    a.kxt = (const T *)h->kxt;
    a.kyt = (const T *)h->kyt;
    set_side<T>(a, h->rowp, ny);
    a.sc = h->sc;
    a.energy = h->energy;
    if (h->lin) {
        table<T>().lintab<<<1024, 256, 0, h->stream>>>((cpx<T> *)h->lin, nx, ny, h->nt, lin_coef(p));
        CK(h, cudaGetLastError());
        a.lintab = (const cpx<T> *)h->lin;
    }

    // Opt in to large dynamic shared memory where needed.
    const KernelTable<T> &K = table<T>();
    struct {
        const void *fn;
        size_t smem;
    } ks[] = {{(const void *)K.row[h->lognx][h->rowv == ROWV_TMA ? 0 : h->rowv],
               K.row_shape[h->lognx][h->rowv == ROWV_TMA ? 0 : h->rowv].smem},
              {(const void *)K.row_tma[h->lognx], K.row_tma_shape[h->lognx].smem},
              {(const void *)K.col[h->logny][h->colv][0], K.col_shape[h->logny][h->colv].smem},
              {(const void *)K.col[h->logny][h->colv][1], K.col_shape[h->logny][h->colv].smem},
              {(const void *)K.col[h->logny][h->colv][2], K.col_shape[h->logny][h->colv].smem},
              {(const void *)K.col[h->logny][h->colv][3], K.col_shape[h->logny][h->colv].smem},
              {(const void *)K.col[h->logny][h->colv][4], K.col_shape[h->logny][h->colv].smem},
              {(const void *)K.rowfwd[h->lognx], K.rowfwd_shape[h->lognx].smem},
              {(const void *)K.colfwd[h->logny], K.colfwd_shape[h->logny].smem}};
    for (auto &k : ks) {
        if (k.fn && k.smem > 48 * 1024)
            CK(h, cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem));
    }
    return AM_OK;
}

// cuTensorMapEncodeTiled from the driver, found through the runtime (the
// library links no driver library of its own).
using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiled encode_tiled()
{
    static EncodeTiled fn = []() -> EncodeTiled {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return reinterpret_cast<EncodeTiled>(p);
    }();
    return fn;
}

namespace af {
// A tensor map of FP32 tiled fields for the row pass: {8 floats of a tile row,
// Ny rows, nt column tiles, nfields fields field_stride bytes apart}, boxes of
// one row and `box` tiles of one field.  False if the encoder is unavailable
// or refuses the geometry.
bool encode_row_map(TmaDesc *out, void *base, int ny, int nt, int nfields, size_t field_stride, int box)
{
    EncodeTiled enc = encode_tiled();
    if (!enc) return false;
    static_assert(sizeof(CUtensorMap) == sizeof(TmaDesc) && alignof(TmaDesc) >= alignof(CUtensorMap),
                  "TmaDesc holds a CUtensorMap");
    const int W = Tile<float>::W;
    const cuuint64_t row_bytes = (cuuint64_t)(2 * W) * sizeof(float);
    const cuuint64_t dims[4] = {(cuuint64_t)(2 * W), (cuuint64_t)ny, (cuuint64_t)nt, (cuuint64_t)nfields};
    const cuuint64_t strides[3] = {row_bytes, row_bytes * ny, (cuuint64_t)field_stride};
    const cuuint32_t boxd[4] = {(cuuint32_t)(2 * W), 1, (cuuint32_t)box, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    return enc(reinterpret_cast<CUtensorMap *>(out), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims, strides, boxd,
               estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
}  // namespace af

// Tensor maps of the FP32 row pass's three inputs (fy, fx, fa) for the
// handle's current pruning: each field as {8 floats of a tile row, Ny rows,
// column tiles, 1 field}, boxes of one row and `box` tiles, nbox boxes per row covering
// the ntp carried tiles (a box may run past them: those tiles are read and
// never used).  tma_ok only where those tiles fit one exchange
// buffer of the row pass (else row shape 2 runs as shape 0).
static void prepare_row_tma(am_handle *h)
{
    h->tma_ok = false;
    if (h->prec != AM_FP32 || h->rowv != ROWV_TMA) return;
    const KernelTable<float> &K = kernels_f32();
    const StepArgs<float> &a = h->a32;
    if (!K.row_tma[h->lognx]) return;
    const int W = Tile<float>::W;
    // boxes of a multiple of 4 tiles (128 bytes), so that every box lands on
    // a 128-byte boundary of the staging buffer
    const int nbox = (a.ntp + 255) / 256, box = ((a.ntp + nbox - 1) / nbox + 3) / 4 * 4;
    if (nbox * box * W > K.row_tma_cap[h->lognx]) return;
    const size_t field_bytes = (size_t)2 * W * sizeof(float) * h->p.ny * h->nt;
    void *fields[3] = {h->fy, h->fx, h->fa};
    for (int f = 0; f < 3; f++)
        if (!encode_row_map(&h->tma.map[f], fields[f], h->p.ny, h->nt, 1, field_bytes, box)) return;
    h->tma.nbox = nbox;
    h->tma.box = box;
    h->tma.shared = 0;
    h->tma_ok = true;
}

template <typename T>
static am_status launch_col(am_handle *h, int mode)
{
    const KernelTable<T> &K = table<T>();
    StepArgs<T> a = args_of<T>(h);
    a.mode = mode;
    const LaunchShape &s = K.col_shape[h->logny][h->colv];
    int grid = col_grid(s, a.ntp, Tile<T>::W);
    K.col[h->logny][h->colv][mode]<<<grid, s.threads, s.smem, h->stream>>>(a);
    CK(h, cudaGetLastError());
    return AM_OK;
}

template <typename T>
static am_status launch_row(am_handle *h)
{
    const KernelTable<T> &K = table<T>();
    if (h->rowv == ROWV_TMA) {
        if constexpr (std::is_same_v<T, float>) {
            prepare_row_tma(h);
            if (h->tma_ok) {
                const LaunchShape &s = K.row_tma_shape[h->lognx];
                int grid = (h->p.ny + s.per_block - 1) / s.per_block;
                K.row_tma[h->lognx]<<<grid, s.threads, s.smem, h->stream>>>(args_of<T>(h), h->tma);
                CK(h, cudaGetLastError());
                return AM_OK;
            }
        }
    }
    const int v = h->rowv == ROWV_TMA ? 0 : h->rowv;   // shape 2 without usable maps runs as shape 0
    const LaunchShape &s = K.row_shape[h->lognx][v];
    int grid = (h->p.ny + s.per_block - 1) / s.per_block;
    K.row[h->lognx][v]<<<grid, s.threads, s.smem, h->stream>>>(args_of<T>(h));
    CK(h, cudaGetLastError());
    return AM_OK;
}

template <typename T>
static am_status enqueue_step(am_handle *h)
{
    for (int s = 1; s <= 4; s++) {
        am_status st = launch_row<T>(h);
        if (st) return st;
        st = launch_col<T>(h, s);
        if (st) return st;
    }
    return AM_OK;
}

template <typename T>
static am_status build_graph(am_handle *h)
{
    if (h->graph) return AM_OK;
    cudaGraph_t g;
    CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    am_status st = enqueue_step<T>(h);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (st) return st;
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaGraphInstantiate");
    return AM_OK;
}

// The four row passes of a step alone, as a graph (am_row_passes_async).
template <typename T>
static am_status build_rows_graph(am_handle *h)
{
    if (h->graph_rows) return AM_OK;
    cudaGraph_t g;
    CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    am_status st = AM_OK;
    for (int s = 1; s <= 4 && !st; s++) st = launch_row<T>(h);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (st) return st;
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&h->graph_rows, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaGraphInstantiate");
    return AM_OK;
}

static am_status reset_scalars(am_handle *h, const double mean[2])
{
    Scalars s{};
    s.m_new[0] = mean ? mean[0] : 0.0;
    s.m_new[1] = mean ? mean[1] : 0.0;
    s.m_old[0] = s.m_appr[0] = s.m_new[0];
    s.m_old[1] = s.m_appr[1] = s.m_new[1];
    s.step = 0;
    s.nan_step = -1;
    CK(h, cudaMemcpyAsync(h->sc, &s, sizeof(s), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return AM_OK;
}

// Select pruned transforms when the 1/2 rule is on and the state is zero
// outside its ellipse; the step graph bakes the launch shape in, so it is
// rebuilt when the choice changes.
template <typename T>
static void choose_pruning(am_handle *h, bool on)
{
    StepArgs<T> &a = args_of<T>(h);
    const int old = a.ntp;
    set_pruning<T>(a, on && h->p.dealias == AM_DEALIAS_HALF);
    if (a.ntp != old && h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    if (a.ntp != old && h->graph_rows) {
        cudaGraphExecDestroy(h->graph_rows);
        h->graph_rows = nullptr;
    }
}

template <typename T>
static am_status set_state_impl(am_handle *h, const void *w_hat, const double mean[2])
{
    const size_t bytes = (size_t)h->p.ny * h->nxh * sizeof(cpx<T>);
    CK(h, cudaMemcpyAsync(h->stage, w_hat, bytes, cudaMemcpyHostToDevice, h->stream));
    if constexpr (std::is_same_v<T, df>) df_from_double_async(h->stage, (size_t)2 * h->p.ny * h->nxh, h->stream);
    am_status st = reset_scalars(h, mean);   // (zeroes Scalars::outside)
    if (st) return st;
    // Pruned transforms need a state that is zero outside the 1/2-rule
    // ellipse: the tile kernel checks that on the device while it converts
    // the layout, and the choice is made before the first column pass.
    const bool half = h->p.dealias == AM_DEALIAS_HALF;
    table<T>().tile<<<1024, 256, 0, h->stream>>>((const cpx<T> *)h->stage, (cpx<T> *)h->u0, h->p.ny, h->nxh,
                                                 h->nt, h->p.nx, half ? &h->sc->outside : nullptr);
    CK(h, cudaGetLastError());
    int outside = 0;
    if (half) {
        CK(h, cudaMemcpyAsync(&outside, &h->sc->outside, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
    }
    choose_pruning<T>(h, half && outside == 0);
    st = launch_col<T>(h, 0);
    if (st) return st;
    CK(h, cudaStreamSynchronize(h->stream));
    h->state_loaded = true;
    return AM_OK;
}

template <typename T>
static am_status set_state_real_impl(am_handle *h, const void *w_real, const double mean[2], int mask)
{
    choose_pruning<T>(h, mask != 0);
    const KernelTable<T> &K = table<T>();
    const size_t bytes = (size_t)h->p.ny * h->p.nx * sizeof(T);
    CK(h, cudaMemcpyAsync(h->stage, w_real, bytes, cudaMemcpyHostToDevice, h->stream));
    if constexpr (std::is_same_v<T, df>) df_from_double_async(h->stage, (size_t)h->p.ny * h->p.nx, h->stream);
    const LaunchShape &rs = K.rowfwd_shape[h->lognx];
    K.rowfwd[h->lognx]<<<(h->p.ny + rs.per_block - 1) / rs.per_block, rs.threads, rs.smem, h->stream>>>(
        (const T *)h->stage, (cpx<T> *)h->P, (const cpx<T> *)h->twx, h->p.ny, h->nt);
    CK(h, cudaGetLastError());
    const LaunchShape &cs = K.colfwd_shape[h->logny];
    K.colfwd[h->logny]<<<(h->nt + cs.per_block - 1) / cs.per_block, cs.threads, cs.smem, h->stream>>>(
        (const cpx<T> *)h->P, (cpx<T> *)h->u0, (const cpx<T> *)h->twy, h->p.nx, h->p.ny, h->nxh, h->nt, mask,
        h->p.dealias, args_of<T>(h).rsq);
    CK(h, cudaGetLastError());
    am_status st = reset_scalars(h, mean);
    if (st) return st;
    st = launch_col<T>(h, 0);
    if (st) return st;
    CK(h, cudaStreamSynchronize(h->stream));
    h->state_loaded = true;
    return AM_OK;
}

template <typename T>
static am_status get_state_impl(am_handle *h, void *w_hat, double mean[2])
{
    table<T>().untile<<<1024, 256, 0, h->stream>>>((const cpx<T> *)h->u0, (cpx<T> *)h->stage, h->p.ny, h->nxh,
                                                   h->nt);
    CK(h, cudaGetLastError());
    if constexpr (std::is_same_v<T, df>) {
        df_to_double_async(h->stage, (size_t)2 * h->p.ny * h->nxh, h->stream);
        CK(h, cudaGetLastError());
    }
    const size_t bytes = (size_t)h->p.ny * h->nxh * sizeof(cpx<T>);
    if (w_hat) CK(h, cudaMemcpyAsync(w_hat, h->stage, bytes, cudaMemcpyDeviceToHost, h->stream));
    Scalars s;
    CK(h, cudaMemcpyAsync(&s, h->sc, sizeof(s), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    if (mean) {
        mean[0] = s.m_new[0];
        mean[1] = s.m_new[1];
    }
    return AM_OK;
}

template <typename T>
static am_status step_impl(am_handle *h, int nsteps, double *energy, int *nan_step, bool wait)
{
    if (nan_step) *nan_step = -1;
    am_status st = build_graph<T>(h);
    if (st) return st;
    if (!wait) {
        for (int i = 0; i < nsteps; i++) CK(h, cudaGraphLaunch(h->graph, h->stream));
        return AM_OK;
    }
    int done = 0;
    while (done < nsteps) {
        int k = nsteps - done < ECAP ? nsteps - done : ECAP;
        CK(h, cudaMemsetAsync(&h->sc->step, 0, sizeof(int), h->stream));
        for (int i = 0; i < k; i++) CK(h, cudaGraphLaunch(h->graph, h->stream));
        if (energy)
            CK(h, cudaMemcpyAsync(energy + done, h->energy, k * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        Scalars s;
        CK(h, cudaMemcpyAsync(&s, h->sc, sizeof(s), cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
        if (s.nan_step >= 0) {
            if (nan_step) *nan_step = done + s.nan_step;
            h->err = "w(0,0) is NaN after step " + std::to_string(done + s.nan_step);
            return AM_ERR_NAN;
        }
        if (s.status != 0) {
            h->err = "a row pass's tensor-map copies did not complete in time";
            return AM_ERR_TIMEOUT;
        }
        done += k;
    }
    return AM_OK;
}

// ------------------------------------------------ column-pass launch shapes

namespace af {

namespace {
// [precision][log2 Ny]: 0 wide, 1 narrow, 2 wide radix 8; seeded with the measured rule
std::atomic<int> g_colv[3][LOG_MAX + 1] = {
    {{1}, {1}, {1}, {1}, {1}, {1}, {1}, {1}, {1}, {1}, {1}, {0}, {0}},
    {{1}, {1}, {1}, {1}, {1}, {1}, {1}, {1}, {1}, {1}, {1}, {0}, {0}},
    {{1}, {1}, {1}, {1}, {1}, {1}, {1}, {1}, {1}, {1}, {1}, {0}, {0}}};
static_assert(LOG_MAX == 12, "seed table covers log2 Ny = 0..12");
int pidx(int prec) { return prec == AM_FP64 ? 1 : prec == AM_DF64 ? 2 : 0; }
}  // namespace

int col_variant(int prec, int logny) { return g_colv[pidx(prec)][logny].load(std::memory_order_relaxed); }
void set_col_variant(int prec, int logny, int v) { g_colv[pidx(prec)][logny].store(v); }

// True if column-pass shape v is built for this precision and log2 Ny: wide
// radix 8 is FP32 only; double-float has the seeded shape of each length only.
bool col_variant_built(int prec, int logny, int v)
{
    if (v < 0 || v >= NCOLV) return false;
    if (prec == AM_DF64) return v == (logny < 11 ? 1 : 0);
    return !(prec == AM_FP64 && v == 2);
}

namespace {
// [precision][log2 Nx]: 0 lockstep radix 8, 1 in sequence with stashes, 2
// lockstep with tensor-map row fetches; seeded with 0, except FP32 from 1024
// (shape 2: 8-15% faster row passes on GB300 at 1024-4096; at 128-512 the
// two are even or shape 0 ahead) and double-float from Nx = 1024 (shape 1:
// the lockstep kernel outgrows the instruction caches)
std::atomic<int> g_rowv[3][LOG_MAX + 1] = {
    {{0}, {0}, {0}, {0}, {0}, {0}, {0}, {0}, {0}, {0}, {2}, {2}, {2}},
    {},
    {{0}, {0}, {0}, {0}, {0}, {0}, {0}, {0}, {0}, {0}, {1}, {1}, {1}}};
}  // namespace

int row_variant(int prec, int lognx) { return g_rowv[pidx(prec)][lognx].load(std::memory_order_relaxed); }
void set_row_variant(int prec, int lognx, int v) { g_rowv[pidx(prec)][lognx].store(v); }
// In sequence with stashes: FP32 and double-float, Nx >= 1024.  Tensor-map
// row fetches: FP32, Nx >= 128.
bool row_variant_built(int prec, int lognx, int v)
{
    if (v == ROWV_TMA) return prec == AM_FP32 && lognx >= 7 && lognx <= LOG_MAX;
    return v == 0 || (v == 1 && prec != AM_FP64 && lognx >= ROWS_LOG_MIN && lognx <= LOG_MAX);
}

}  // namespace af

// Switch a handle to column-pass shape v (kernel attributes, step graph).
template <typename T>
static am_status use_col_variant(am_handle *h, int v)
{
    const KernelTable<T> &K = table<T>();
    const LaunchShape &cs = K.col_shape[h->logny][v];
    for (int m = 0; m < 5; m++)
        if (cs.smem > 48 * 1024)
            CK(h, cudaFuncSetAttribute((const void *)K.col[h->logny][v][m],
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cs.smem));
    if (h->colv != v && h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    h->colv = v;
    return AM_OK;
}

// Switch a handle to row-pass shape v (kernel attribute, step graphs).
template <typename T>
static am_status use_row_variant(am_handle *h, int v)
{
    const KernelTable<T> &K = table<T>();
    const int v0 = v == ROWV_TMA ? 0 : v;   // shape 2 falls back to shape 0's kernel
    const LaunchShape &rs = K.row_shape[h->lognx][v0];
    if (rs.smem > 48 * 1024)
        CK(h, cudaFuncSetAttribute((const void *)K.row[h->lognx][v0], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)rs.smem));
    if (v == ROWV_TMA && K.row_tma[h->lognx] && K.row_tma_shape[h->lognx].smem > 48 * 1024)
        CK(h, cudaFuncSetAttribute((const void *)K.row_tma[h->lognx], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)K.row_tma_shape[h->lognx].smem));
    if (h->rowv != v) {
        if (h->graph) cudaGraphExecDestroy(h->graph);
        if (h->graph_rows) cudaGraphExecDestroy(h->graph_rows);
        h->graph = nullptr;
        h->graph_rows = nullptr;
    }
    h->rowv = v;
    return AM_OK;
}

// ------------------------------------------- serving-engine hooks (internal)

namespace af {

int handle_ring_capacity() { return ECAP; }

cudaStream_t handle_stream(const am_handle *h) { return h ? h->stream : nullptr; }

am_status handle_enqueue_chunk(am_handle *h, int k, double *energy_host, void *scalars_host, cudaEvent_t done)
{
    if (!h || k < 1 || k > ECAP || !scalars_host || !h->state_loaded) return AM_ERR_ARG;
    am_status st = with_type(h->prec, [&](auto t) { return build_graph<decltype(t)>(h); });
    if (st) return st;
    CK(h, cudaMemsetAsync(&h->sc->step, 0, sizeof(int), h->stream));
    for (int i = 0; i < k; i++) CK(h, cudaGraphLaunch(h->graph, h->stream));
    if (energy_host)
        CK(h, cudaMemcpyAsync(energy_host, h->energy, k * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(scalars_host, h->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaEventRecord(done, h->stream));
    return AM_OK;
}

}  // namespace af

// ------------------------------------------------------------------- C ABI

extern "C" {

const char *am_status_string(am_status s)
{
    switch (s) {
    case AM_OK: return "ok";
    case AM_ERR_ARG: return "invalid argument";
    case AM_ERR_CUDA: return "CUDA error";
    case AM_ERR_NAN: return "array contains nan values";
    case AM_ERR_IO: return "I/O error";
    case AM_ERR_SPEC: return "specification error";
    case AM_ERR_OOM: return "out of device memory";
    case AM_ERR_UNSUPPORTED: return "unsupported";
    case AM_ERR_TIMEOUT: return "timed out";
    }
    return "unknown status";
}

const char *am_last_error(const am_handle *h) { return h ? h->err.c_str() : ""; }

int am_mask_value(int nx, int ny, int dealias, int ix, int iy)
{
    return mask_at(dealias, reference_rsq(nx, ny), nx, ny, ix, iy);
}

am_status am_create(const am_params *p, am_handle **out)
{
    if (!p || !out) return AM_ERR_ARG;
    *out = nullptr;
    if (!is_pow2(p->nx) || !is_pow2(p->ny) || p->nx < (1 << LOG_MIN) || p->ny < (1 << LOG_MIN) ||
        p->nx > (1 << LOG_MAX) || p->ny > (1 << LOG_MAX))
        return AM_ERR_UNSUPPORTED;
    if (p->precision != AM_FP32 && p->precision != AM_FP64 && p->precision != AM_DF64) return AM_ERR_ARG;
    if (p->dealias < 0 || p->dealias > 2 || (p->form != AM_FORM_REFERENCE && p->form != AM_FORM_GENERAL))
        return AM_ERR_ARG;
    if (!(p->lx > 0) || !(p->ly > 0) || !std::isfinite(p->dt)) return AM_ERR_ARG;
    if (p->if_factors < AM_IF_AUTO || p->if_factors > AM_IF_DOUBLE) return AM_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return AM_ERR_CUDA;
    am_handle *h = new (std::nothrow) am_handle();
    if (!h) return AM_ERR_OOM;
    h->p = *p;
    h->prec = p->precision;
    h->lognx = ilog2(p->nx);
    h->logny = ilog2(p->ny);
    h->colv = col_variant(h->prec, h->logny);
    h->rowv = row_variant(h->prec, h->lognx);
    cudaGetDevice(&h->device);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return AM_ERR_CUDA;
    }
    h->own_stream = true;
    am_status st = with_type(h->prec, [&](auto t) { return alloc_and_tables<decltype(t)>(h); });
    if (st) {
        am_destroy(h);
        return st;
    }
    *out = h;
    return AM_OK;
}

am_status am_destroy(am_handle *h)
{
    if (!h) return AM_OK;
    if (h->graph) cudaGraphExecDestroy(h->graph);
    if (h->graph_rows) cudaGraphExecDestroy(h->graph_rows);
    // Stream-ordered frees: the memory returns to the pool once the handle's
    // own work is done, without waiting for other streams of the device.
    void *ptrs[] = {h->u0, h->acc, h->fa, h->fx, h->fy, h->P, h->Q, h->stage, h->twx, h->twy,
                    h->kxt, h->kyt, h->lin, h->rowp, h->energy, h->sc};
    for (void *q : ptrs)
        if (q) cudaFreeAsync(q, h->stream);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return AM_OK;
}

am_status am_set_stream(am_handle *h, void *stream)
{
    if (!h) return AM_ERR_ARG;
    CK(h, cudaStreamSynchronize(h->stream));
    if (h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    if (h->graph_rows) {
        cudaGraphExecDestroy(h->graph_rows);
        h->graph_rows = nullptr;
    }
    if (stream) {
        if (h->own_stream) cudaStreamDestroy(h->stream);
        h->own_stream = false;
        h->stream = (cudaStream_t)stream;
    } else if (!h->own_stream) {
        CK(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->own_stream = true;
    }
    return AM_OK;
}

am_status am_set_state(am_handle *h, const void *w_hat, const double mean[2])
{
    if (!h || !w_hat) return AM_ERR_ARG;
    return with_type(h->prec, [&](auto t) { return set_state_impl<decltype(t)>(h, w_hat, mean); });
}

am_status am_set_state_real(am_handle *h, const void *w_real, const double mean[2], int mask_and_zero_mean)
{
    if (!h || !w_real) return AM_ERR_ARG;
    return with_type(h->prec,
                     [&](auto t) { return set_state_real_impl<decltype(t)>(h, w_real, mean, mask_and_zero_mean); });
}

am_status am_get_state(am_handle *h, void *w_hat, double mean[2])
{
    if (!h) return AM_ERR_ARG;
    if (!h->state_loaded) {
        h->err = "no state loaded";
        return AM_ERR_ARG;
    }
    return with_type(h->prec, [&](auto t) { return get_state_impl<decltype(t)>(h, w_hat, mean); });
}

am_status am_step(am_handle *h, int nsteps, double *energy, int *nan_step)
{
    if (!h || nsteps < 0) return AM_ERR_ARG;
    if (!h->state_loaded) {
        h->err = "no state loaded";
        return AM_ERR_ARG;
    }
    return with_type(h->prec, [&](auto t) { return step_impl<decltype(t)>(h, nsteps, energy, nan_step, true); });
}

am_status am_step_async(am_handle *h, int nsteps)
{
    if (!h || nsteps < 0) return AM_ERR_ARG;
    if (!h->state_loaded) return AM_ERR_ARG;
    return with_type(h->prec, [&](auto t) { return step_impl<decltype(t)>(h, nsteps, nullptr, nullptr, false); });
}

am_status am_sync(am_handle *h)
{
    if (!h) return AM_ERR_ARG;
    Scalars s;
    CK(h, cudaMemcpyAsync(&s, h->sc, sizeof(s), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    if (s.nan_step >= 0) return AM_ERR_NAN;
    return AM_OK;
}

am_status am_step_profiled(am_handle *h, int nsteps, double row_ms[4], double col_ms[4])
{
    if (!h || nsteps < 0 || !row_ms || !col_ms) return AM_ERR_ARG;
    if (!h->state_loaded) return AM_ERR_ARG;
    // One step captured as a graph with a timing event before and after each
    // of the 8 kernels (external event-record nodes), so the kernels run as in
    // the production graph: back to back, no host work between them.
    cudaEvent_t ev[9] = {};
    for (auto &e : ev) CK(h, cudaEventCreate(&e));
    am_status st = AM_OK;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    cudaError_t ce = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
    if (ce != cudaSuccess) st = cuda_fail(h, ce, "cudaStreamBeginCapture");
    if (!st) {
        ce = cudaEventRecordWithFlags(ev[0], h->stream, cudaEventRecordExternal);
        for (int s = 1; s <= 4 && !st && ce == cudaSuccess; s++) {
            st = with_type(h->prec, [&](auto t) { return launch_row<decltype(t)>(h); });
            if (!st) ce = cudaEventRecordWithFlags(ev[2 * s - 1], h->stream, cudaEventRecordExternal);
            if (!st && ce == cudaSuccess)
                st = with_type(h->prec, [&](auto t) { return launch_col<decltype(t)>(h, s); });
            if (!st && ce == cudaSuccess) ce = cudaEventRecordWithFlags(ev[2 * s], h->stream, cudaEventRecordExternal);
        }
        cudaError_t ee = cudaStreamEndCapture(h->stream, &g);
        if (!st && ce != cudaSuccess) st = cuda_fail(h, ce, "cudaEventRecordWithFlags");
        if (!st && ee != cudaSuccess) st = cuda_fail(h, ee, "cudaStreamEndCapture");
    }
    if (!st) {
        ce = cudaGraphInstantiate(&ge, g, 0);
        if (ce != cudaSuccess) st = cuda_fail(h, ce, "cudaGraphInstantiate");
    }
    for (int m = 0; m < nsteps && !st; m++) {
        ce = cudaGraphLaunch(ge, h->stream);
        if (ce == cudaSuccess) ce = cudaEventSynchronize(ev[8]);
        if (ce != cudaSuccess) {
            st = cuda_fail(h, ce, "profiled step");
            break;
        }
        for (int s = 1; s <= 4 && !st; s++) {
            float a = 0, b = 0;
            ce = cudaEventElapsedTime(&a, ev[2 * s - 2], ev[2 * s - 1]);
            if (ce == cudaSuccess) ce = cudaEventElapsedTime(&b, ev[2 * s - 1], ev[2 * s]);
            if (ce != cudaSuccess) st = cuda_fail(h, ce, "cudaEventElapsedTime");
            row_ms[s - 1] += a;
            col_ms[s - 1] += b;
        }
    }
    if (ge) cudaGraphExecDestroy(ge);
    if (g) cudaGraphDestroy(g);
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    return st;
}

am_status am_row_passes_async(am_handle *h, int reps)
{
    if (!h || reps < 0) return AM_ERR_ARG;
    if (!h->state_loaded) return AM_ERR_ARG;
    am_status st = with_type(h->prec, [&](auto t) { return build_rows_graph<decltype(t)>(h); });
    if (st) return st;
    for (int i = 0; i < reps; i++) CK(h, cudaGraphLaunch(h->graph_rows, h->stream));
    return AM_OK;
}

am_status am_set_column_shape(int precision, int ny, int shape)
{
    if (!is_pow2(ny) || ny < (1 << LOG_MIN) || ny > (1 << LOG_MAX) || shape < 0 || shape >= NCOLV ||
        (precision != AM_FP32 && precision != AM_FP64 && precision != AM_DF64))
        return AM_ERR_ARG;
    if (!col_variant_built(precision, ilog2(ny), shape)) return AM_ERR_UNSUPPORTED;
    set_col_variant(precision, ilog2(ny), shape);
    return AM_OK;
}

int am_column_shape(int precision, int ny)
{
    if (!is_pow2(ny) || ny < (1 << LOG_MIN) || ny > (1 << LOG_MAX) ||
        (precision != AM_FP32 && precision != AM_FP64 && precision != AM_DF64))
        return -1;
    return col_variant(precision, ilog2(ny));
}

am_status am_set_row_shape(int precision, int nx, int shape)
{
    if (!is_pow2(nx) || nx < (1 << LOG_MIN) || nx > (1 << LOG_MAX) || shape < 0 || shape >= NROWV ||
        (precision != AM_FP32 && precision != AM_FP64 && precision != AM_DF64))
        return AM_ERR_ARG;
    if (!row_variant_built(precision, ilog2(nx), shape)) return AM_ERR_UNSUPPORTED;
    set_row_variant(precision, ilog2(nx), shape);
    return AM_OK;
}

int am_row_shape(int precision, int nx)
{
    if (!is_pow2(nx) || nx < (1 << LOG_MIN) || nx > (1 << LOG_MAX) ||
        (precision != AM_FP32 && precision != AM_FP64 && precision != AM_DF64))
        return -1;
    return row_variant(precision, ilog2(nx));
}

// Time nsteps graph replays of the handle's step (after two warm-up steps).
static am_status time_steps(am_handle *h, int nsteps, cudaEvent_t e0, cudaEvent_t e1, double *per)
{
    am_status st = am_step(h, 2, nullptr, nullptr);   // warm-up, builds the graph
    if (st) return st;
    CK(h, cudaEventRecord(e0, h->stream));
    for (int i = 0; i < nsteps; i++) CK(h, cudaGraphLaunch(h->graph, h->stream));
    float ms = 0;
    CK(h, cudaEventRecord(e1, h->stream));
    CK(h, cudaEventSynchronize(e1));
    CK(h, cudaEventElapsedTime(&ms, e0, e1));
    *per = (double)ms / nsteps;
    return AM_OK;
}

am_status am_autotune(const am_params *p, int nsteps, double ms_col[3], double ms_row[3])
{
    if (!p || nsteps < 1) return AM_ERR_ARG;
    am_handle *h = nullptr;
    am_status st = am_create(p, &h);
    if (st) return st;
    // a seeded band-limited state in the handle's precision
    const size_t n = (size_t)p->ny * (p->nx / 2 + 1) * 2;
    std::vector<double> w(n);
    st = am_ic_bandlimited(p->nx, p->ny, 1, 1.0, 8.0, 0.01, w.data());
    std::vector<float> wf;
    if (!st && p->precision == AM_FP32) {
        wf.resize(n);
        for (size_t i = 0; i < n; i++) wf[i] = (float)w[i];
    }
    if (!st) st = am_set_state(h, p->precision == AM_FP32 ? (const void *)wf.data() : (const void *)w.data(), nullptr);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!st && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) st = AM_ERR_CUDA;
    // Coordinate search: the column-pass shapes with the current row shape,
    // then the row-pass shapes with the best column shape.
    int bestc = h ? h->colv : 0, bestr = h ? h->rowv : 0;
    double best = 0;
    bool first = true;
    for (int v = 0; v < NCOLV && !st; v++) {
        if (!col_variant_built(h->prec, h->logny, v)) {
            if (ms_col) ms_col[v] = -1;   // not built for this precision
            continue;
        }
        st = with_type(h->prec, [&](auto t) { return use_col_variant<decltype(t)>(h, v); });
        double per = 0;
        if (!st) st = time_steps(h, nsteps, e0, e1, &per);
        if (st) break;
        if (ms_col) ms_col[v] = per;
        if (first || per < best) {
            best = per;
            bestc = v;
            first = false;
        }
    }
    if (!st) st = with_type(h->prec, [&](auto t) { return use_col_variant<decltype(t)>(h, bestc); });
    first = true;
    for (int v = 0; v < NROWV && !st; v++) {
        if (!row_variant_built(h->prec, h->lognx, v)) {
            if (ms_row) ms_row[v] = -1;
            continue;
        }
        st = with_type(h->prec, [&](auto t) { return use_row_variant<decltype(t)>(h, v); });
        double per = 0;
        if (!st) st = time_steps(h, nsteps, e0, e1, &per);
        if (st) break;
        if (ms_row) ms_row[v] = per;
        if (first || per < best) {
            best = per;
            bestr = v;
            first = false;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    am_destroy(h);
    if (!st) {
        set_col_variant(p->precision, ilog2(p->ny), bestc);
        set_row_variant(p->precision, ilog2(p->nx), bestr);
    }
    return st;
}

int am_launches_per_step(const am_handle *h) { return h ? 8 : 0; }

long long am_device_bytes(const am_handle *h) { return h ? h->bytes : 0; }

long long am_footprint_bytes(const am_params *p)
{
    if (!p || !is_pow2(p->nx) || !is_pow2(p->ny)) return -1;
    const bool f64 = p->precision != AM_FP32;   // FP64 and double-float: 8-byte reals
    const size_t cs = f64 ? sizeof(cpx<double>) : sizeof(cpx<float>), rs = f64 ? sizeof(double) : sizeof(float);
    const int W = f64 ? Tile<double>::W : Tile<float>::W;
    const int nxh = p->nx / 2 + 1, nt = (nxh + W - 1) / W;
    const size_t field = (size_t)nt * W * p->ny * cs;
    return (long long)((use_if_table(*p) ? 8 : 7) * field + (size_t)p->ny * nxh * cs + (size_t)(p->nx + p->ny) * cs +
                       (size_t)nt * W * rs + (size_t)p->ny * rs + side_bytes(p->ny) + ECAP * sizeof(double) +
                       sizeof(Scalars));
}

int am_kx_carried(const am_handle *h)
{
    if (!h) return -1;
    return h->prec == AM_FP64 ? h->a64.kxp : h->prec == AM_DF64 ? h->adf.kxp : h->a32.kxp;
}

am_status am_ic_bandlimited(int nx, int ny, unsigned long long seed, double kmin, double kmax, double rms,
                            double *w_hat)
{
    if (!w_hat || nx < 4 || ny < 4 || kmax < 0 || 2 * kmax >= nx || 2 * kmax >= ny) return AM_ERR_ARG;
    const int nxh = nx / 2 + 1;
    std::memset(w_hat, 0, sizeof(double) * 2 * (size_t)ny * nxh);
    std::mt19937_64 gen(seed);
    auto unit = [&gen]() { return (double)(gen() >> 11) * (1.0 / 9007199254740992.0); };
    const int km = (int)std::floor(kmax);
    const double kmin2 = kmin * kmin, kmax2 = kmax * kmax;
    for (int iy = -km; iy <= km; iy++) {
        for (int ix = 0; ix <= km; ix++) {
            if (ix == 0 && iy <= 0) continue;
            double r2 = (double)(ix * ix + iy * iy);
            if (r2 < kmin2 || r2 > kmax2) continue;
            double u1 = unit(), u2 = unit(), u3 = unit();
            double amp = std::sqrt(-2.0 * std::log(1.0 - u1)) * std::cos(2.0 * M_PI * u2);
            double ph = 2.0 * M_PI * u3;
            double re = amp * std::cos(ph), im = amp * std::sin(ph);
            size_t k = ((size_t)((iy % ny + ny) % ny) * nxh + ix) * 2;
            w_hat[k] = re;
            w_hat[k + 1] = im;
            if (ix == 0) {
                size_t kc = ((size_t)((-iy % ny + ny) % ny) * nxh) * 2;
                w_hat[kc] = re;
                w_hat[kc + 1] = -im;
            }
        }
    }
    // Scale to the requested real-space rms (Parseval on the full plane).
    double full = 0;
    for (int iy = 0; iy < ny; iy++)
        for (int ix = 0; ix < nxh; ix++) {
            size_t k = ((size_t)iy * nxh + ix) * 2;
            double a2 = w_hat[k] * w_hat[k] + w_hat[k + 1] * w_hat[k + 1];
            full += (ix == 0 ? 1.0 : 2.0) * a2;
        }
    double cur = std::sqrt(full) / ((double)nx * ny);
    if (cur > 0) {
        double f = rms / cur;
        for (size_t k = 0; k < (size_t)2 * ny * nxh; k++) w_hat[k] *= f;
    }
    return AM_OK;
}

}  // extern "C"
