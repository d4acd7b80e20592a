// Ragged batches: simulations of different grid sizes, parameters, time
// steps and step counts advanced together.
//
// The reference runs one simulation per process (its time loop,
// ActFlow_V3-2.cu:718-862); a ragged batch is that loop for R independent
// runs at once.  Runs are grouped into size classes (same Nx, Ny), the work
// list is sorted by grid size (largest class first), and each pass of a step
// is ONE launch per class covering all of its active runs (blockIdx.y = run
// within the class, the same batched kernels as ensembles).  A step is one
// CUDA graph whose classes are parallel branches (forked capture streams), so
// the small grids' launches fill the SMs the large grids leave idle.
//
// Work-list mode (am_ragged_set_mode): instead of one launch per
// class, each pass of a stage is ONE launch over a work list of (run, CTA)
// items of every class, sorted by grid size, largest first; each CTA runs the
// kernel body of its item's length (kernels_queue.cu).  A step is then 8
// launches whatever the number of classes, and the block scheduler hands out
// the large grids' long items first.  It uses the radix-8 row pass and the
// narrow column pass for every class (the shapes whose CTAs have 128 threads
// at every length); the per-class mode (the default) uses each class's tuned
// shapes, and measured faster on GB300 (40-run batch: 1.78e10 against 1.27e10
// grid-point-steps/s, the radix-8 column shape winning at every size).
//
// Runs stop at their own step counts: the batch advances in segments of
// k = min(remaining steps over the active runs, energy-ring capacity) steps;
// after a segment the finished runs are dropped from the per-class argument
// arrays and the graph is rebuilt for the remaining active set (at most one
// rebuild per distinct step count).  No kernel waits on another: ordering
// comes from the graph's edges only.
//
// Each run computes exactly what a lone handle with its parameters computes
// (the same kernel bodies and arguments; pruned and full transforms give the
// same values).  FP32, grids 128..1024 per axis.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "actflow.h"
#include "host_tables.h"
#include "kernels.h"

using namespace af;

namespace {
constexpr int ECAP_R = 1024;   // energy ring entries per run
constexpr size_t ALIGN = 256;

size_t align_up(size_t n) { return (n + ALIGN - 1) / ALIGN * ALIGN; }

int ilog2_exact(int n)
{
    int l = 0;
    while ((1 << l) < n) l++;
    return (1 << l) == n ? l : -1;
}

__global__ void k_ragged_reset_steps(Scalars *sc, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) sc[i].step = 0;
}

struct RaggedRun {
    am_params p{};
    long long nsteps = 0, done = 0;
    int cls = -1;
    int nxh = 0, nt = 0;
    size_t field_elems = 0;
    size_t offset = 0;          // byte offset of this run's block in the pool
    StepArgs<float> a{};
    bool loaded = false, inside = false;
};

struct SizeClass {
    int lognx = 0, logny = 0;
    int colv = 0;               // column-pass launch shape (0 wide, 1 narrow, 2 wide radix 8)
    int rowv = 0;               // row-pass launch shape (0 radix 8, 1 radix 16 with stashes)
    std::vector<int> runs;      // run indices of this class
    std::vector<int> active;    // active runs (graph order)
    int ntp = 0;                // column tiles the passes touch (pruned or full)
    int off = 0;                // offset of this class's arguments in dargs
    cudaStream_t branch = nullptr;
    cudaEvent_t joined = nullptr;
};

// Bytes of one run's device block: 7 fields, side buffer, tables, energy
// ring, scalars, each 256-byte aligned.
struct RunLayout {
    size_t fields, lin, side, twx, twy, kx, ky, energy, sc, total;
    bool has_lin;   // integrating-factor table (AM_IF_DOUBLE), one field
};
RunLayout run_layout(const am_params &p)
{
    const int W = Tile<float>::W;
    const int nxh = p.nx / 2 + 1, nt = (nxh + W - 1) / W;
    RunLayout L{};
    size_t o = 0;
    L.fields = o;
    o += align_up(7 * (size_t)nt * W * p.ny * sizeof(cpx<float>));
    L.lin = o;
    L.has_lin = use_if_table(p);
    if (L.has_lin) o += align_up((size_t)nt * W * p.ny * sizeof(cpx<float>));
    L.side = o;
    o += align_up(side_bytes(p.ny));
    L.twx = o;
    o += align_up((size_t)p.nx * sizeof(cpx<float>));
    L.twy = o;
    o += align_up((size_t)p.ny * sizeof(cpx<float>));
    L.kx = o;
    o += align_up((size_t)nt * W * sizeof(float));
    L.ky = o;
    o += align_up((size_t)p.ny * sizeof(float));
    L.energy = o;
    o += align_up(ECAP_R * sizeof(double));
    L.sc = o;
    o += align_up(sizeof(Scalars));
    L.total = o;
    return L;
}

}  // namespace

struct am_ragged {
    std::vector<RaggedRun> runs;
    std::vector<SizeClass> cls;
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr;
    unsigned char *pool = nullptr;
    size_t pool_bytes = 0;
    cpx<float> *stage = nullptr;
    Scalars *sc_all = nullptr;        // scalars of every run, contiguous (reset kernel)
    double *ering_all = nullptr;      // energy rings [nruns][ECAP_R]
    StepArgs<float> *dargs = nullptr;
    int mode = 0;                     // 0: one launch per class per pass; 1: per pass over the work list
    WorkItem *items = nullptr;        // device work lists: rows, then columns
    size_t item_cap = 0;              // capacity of each list
    cudaGraphExec_t graph = nullptr;
    int graph_mode = -1;
    std::vector<char> graph_set;      // active flags the graph was built for
    std::string err;
};

#define RK(call)                                                                \
    do {                                                                        \
        cudaError_t e_ = (call);                                                \
        if (e_ != cudaSuccess) {                                                \
            r->err = std::string(#call) + ": " + cudaGetErrorString(e_);        \
            return e_ == cudaErrorMemoryAllocation ? AM_ERR_OOM : AM_ERR_CUDA;  \
        }                                                                       \
    } while (0)

namespace {

// Work-list mode: the (run, CTA) items of every active run, classes largest
// first (the order of r->cls), uploaded once per active set; the step graph is
// the 8 work-list launches.  The arguments are already in dargs.
am_status rebuild_worklist(am_ragged *r, const std::vector<char> &act, const KernelTable<float> &K)
{
    const QueueTable &Q = kernels_queue_f32();
    std::vector<WorkItem> rows, cols;
    for (const SizeClass &c : r->cls) {
        const LaunchShape &rs = K.row_shape[c.lognx][0];
        const LaunchShape &cs = K.col_shape[c.logny][1];
        const int rblocks = ((1 << c.logny) + rs.per_block - 1) / rs.per_block;
        const int cblocks = col_grid(cs, c.ntp, Tile<float>::W);
        for (size_t q = 0; q < c.active.size(); q++) {
            for (int b = 0; b < rblocks; b++) rows.push_back({c.off + (int)q, b, c.lognx});
            for (int b = 0; b < cblocks; b++) cols.push_back({c.off + (int)q, b, c.logny});
        }
    }
    if (rows.size() > r->item_cap || cols.size() > r->item_cap) {
        r->err = "work list larger than its buffer";
        return AM_ERR_ARG;
    }
    RK(cudaMemcpyAsync(r->items, rows.data(), rows.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, r->stream));
    RK(cudaMemcpyAsync(r->items + r->item_cap, cols.data(), cols.size() * sizeof(WorkItem), cudaMemcpyHostToDevice,
                       r->stream));
    RK(cudaStreamSynchronize(r->stream));
    cudaGraph_t g;
    RK(cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 1; s <= 4; s++) {
        Q.row<<<(unsigned)rows.size(), 128, Q.row_smem, r->stream>>>(r->dargs, r->items);
        Q.col[s]<<<(unsigned)cols.size(), 128, Q.col_smem, r->stream>>>(r->dargs, r->items + r->item_cap);
    }
    cudaError_t e = cudaGetLastError();
    cudaError_t e2 = cudaStreamEndCapture(r->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        r->err = std::string("capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2);
        if (e2 == cudaSuccess) cudaGraphDestroy(g);
        return AM_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&r->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        r->err = std::string("instantiate: ") + cudaGetErrorString(e);
        return AM_ERR_CUDA;
    }
    r->graph_set = act;
    r->graph_mode = 1;
    return AM_OK;
}

// Upload the per-class argument arrays of the active runs and capture the
// step graph: one branch per class, largest grids first.
am_status rebuild(am_ragged *r, const std::vector<char> &act)
{
    if (r->graph && r->graph_set == act && r->graph_mode == r->mode) return AM_OK;
    if (r->graph) {
        cudaGraphExecDestroy(r->graph);
        r->graph = nullptr;
    }
    std::vector<StepArgs<float>> h(r->runs.size());
    int off = 0;
    for (SizeClass &c : r->cls) {
        c.active.clear();
        bool pruned = true;
        for (int i : c.runs)
            if (act[i]) {
                c.active.push_back(i);
                pruned = pruned && r->runs[i].p.dealias == AM_DEALIAS_HALF && r->runs[i].inside;
            }
        c.off = off;
        for (size_t q = 0; q < c.active.size(); q++) {
            StepArgs<float> a = r->runs[c.active[q]].a;
            set_pruning<float>(a, pruned);
            c.ntp = a.ntp;
            h[off + q] = a;
        }
        off += (int)c.active.size();
    }
    if (off == 0) return AM_OK;
    RK(cudaMemcpyAsync(r->dargs, h.data(), off * sizeof(StepArgs<float>), cudaMemcpyHostToDevice, r->stream));
    RK(cudaStreamSynchronize(r->stream));

    const KernelTable<float> &K = kernels_f32();
    const BatchTable &KB = kernels_batch_f32();
    if (r->mode == 1) return rebuild_worklist(r, act, K);
    cudaGraph_t g;
    RK(cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaEventRecord(r->fork, r->stream);
    for (SizeClass &c : r->cls) {
        if (c.active.empty() || e != cudaSuccess) continue;
        e = cudaStreamWaitEvent(c.branch, r->fork, 0);
        if (e != cudaSuccess) break;
        const LaunchShape &rs = K.row_shape[c.lognx][c.rowv];
        const LaunchShape &cs = K.col_shape[c.logny][c.colv];
        const int ny = 1 << c.logny;
        const int nb = (int)c.active.size();
        const dim3 rgrid((ny + rs.per_block - 1) / rs.per_block, nb);
        const dim3 cgrid(col_grid(cs, c.ntp, Tile<float>::W), nb);
        const StepArgs<float> *args = r->dargs + c.off;
        for (int s = 1; s <= 4; s++) {
            KB.row[c.lognx][c.rowv]<<<rgrid, rs.threads, rs.smem, c.branch>>>(args);
            KB.col[c.logny][c.colv][s]<<<cgrid, cs.threads, cs.smem, c.branch>>>(args);
        }
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(c.joined, c.branch);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(r->stream, c.joined, 0);
    }
    cudaError_t e2 = cudaStreamEndCapture(r->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        r->err = std::string("capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2);
        if (e2 == cudaSuccess) cudaGraphDestroy(g);
        return AM_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&r->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        r->err = std::string("instantiate: ") + cudaGetErrorString(e);
        return AM_ERR_CUDA;
    }
    r->graph_set = act;
    r->graph_mode = 0;
    return AM_OK;
}

}  // namespace

extern "C" {

am_status am_ragged_create(const am_params *params, const long long *nsteps, int nruns, am_ragged **out)
{
    if (!params || !nsteps || !out || nruns < 1) return AM_ERR_ARG;
    *out = nullptr;
    for (int i = 0; i < nruns; i++) {
        const am_params &p = params[i];
        const int lx = ilog2_exact(p.nx), ly = ilog2_exact(p.ny);
        if (lx < BATCH_LOG_MIN || lx > BATCH_LOG_MAX || ly < BATCH_LOG_MIN || ly > BATCH_LOG_MAX)
            return AM_ERR_UNSUPPORTED;
        if (p.precision != AM_FP32) return AM_ERR_UNSUPPORTED;
        if (p.dealias < 0 || p.dealias > 2 || (p.form != AM_FORM_REFERENCE && p.form != AM_FORM_GENERAL))
            return AM_ERR_ARG;
        if (!(p.lx > 0) || !(p.ly > 0) || !(p.dt == p.dt) || nsteps[i] < 0) return AM_ERR_ARG;
        if (p.if_factors < AM_IF_AUTO || p.if_factors > AM_IF_DOUBLE) return AM_ERR_ARG;
    }
    am_ragged *r = new (std::nothrow) am_ragged();
    if (!r) return AM_ERR_OOM;
    auto fail = [&](am_status s) {
        am_ragged_destroy(r);
        return s;
    };
    r->runs.resize(nruns);
    // Size classes, largest grid first (ties: wider first).
    std::map<std::pair<int, int>, int> key;
    std::vector<std::pair<int, int>> keys;
    for (int i = 0; i < nruns; i++) {
        std::pair<int, int> k{ilog2_exact(params[i].nx), ilog2_exact(params[i].ny)};
        if (!key.count(k)) {
            key[k] = 0;
            keys.push_back(k);
        }
    }
    std::sort(keys.begin(), keys.end(), [](const std::pair<int, int> &a, const std::pair<int, int> &b) {
        const int sa = a.first + a.second, sb = b.first + b.second;
        return sa != sb ? sa > sb : a.first > b.first;
    });
    r->cls.resize(keys.size());
    for (size_t c = 0; c < keys.size(); c++) {
        key[keys[c]] = (int)c;
        r->cls[c].lognx = keys[c].first;
        r->cls[c].logny = keys[c].second;
        r->cls[c].colv = col_variant(AM_FP32, keys[c].second);
        r->cls[c].rowv = row_variant(AM_FP32, keys[c].first);
        if (r->cls[c].rowv == ROWV_TMA) r->cls[c].rowv = 0;   // single-handle shape
    }
    size_t total = 0, stage = 0;
    for (int i = 0; i < nruns; i++) {
        RaggedRun &run = r->runs[i];
        run.p = params[i];
        run.nsteps = nsteps[i];
        run.cls = key[{ilog2_exact(run.p.nx), ilog2_exact(run.p.ny)}];
        r->cls[run.cls].runs.push_back(i);
        run.offset = total;
        total += run_layout(run.p).total;
        stage = std::max(stage, (size_t)run.p.ny * (run.p.nx / 2 + 1) * sizeof(cpx<float>));
    }
    r->pool_bytes = total;
    if (cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&r->fork, cudaEventDisableTiming) != cudaSuccess)
        return fail(AM_ERR_CUDA);
    for (SizeClass &c : r->cls)
        if (cudaStreamCreateWithFlags(&c.branch, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&c.joined, cudaEventDisableTiming) != cudaSuccess)
            return fail(AM_ERR_CUDA);
    if (cudaMalloc(&r->pool, total) != cudaSuccess || cudaMalloc(&r->stage, stage) != cudaSuccess ||
        cudaMalloc(&r->sc_all, nruns * sizeof(Scalars)) != cudaSuccess ||
        cudaMalloc(&r->ering_all, (size_t)nruns * ECAP_R * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&r->dargs, nruns * sizeof(StepArgs<float>)) != cudaSuccess)
        return fail(AM_ERR_OOM);
    if (cudaMemsetAsync(r->pool, 0, total, r->stream) != cudaSuccess) return fail(AM_ERR_CUDA);

    for (int i = 0; i < nruns; i++) {
        RaggedRun &run = r->runs[i];
        const RunLayout L = run_layout(run.p);
        unsigned char *base = r->pool + run.offset;
        HostTables<float> t;
        StepArgs<float> &a = run.a;
        host_setup<float>(run.p, t, a, ECAP_R);
        run.nxh = t.nxh;
        run.nt = t.nt;
        run.field_elems = (size_t)t.nt * Tile<float>::W * run.p.ny;
        cpx<float> *f = reinterpret_cast<cpx<float> *>(base + L.fields);
        a.u0 = f;
        a.acc = f + run.field_elems;
        a.fa = f + 2 * run.field_elems;
        a.fx = f + 3 * run.field_elems;
        a.fy = f + 4 * run.field_elems;
        a.P = f + 5 * run.field_elems;
        a.Q = f + 6 * run.field_elems;
        a.twx = reinterpret_cast<const cpx<float> *>(base + L.twx);
        a.twy = reinterpret_cast<const cpx<float> *>(base + L.twy);
        a.kxt = reinterpret_cast<const float *>(base + L.kx);
        a.kyt = reinterpret_cast<const float *>(base + L.ky);
        set_side<float>(a, base + L.side, run.p.ny);
        a.sc = r->sc_all + i;
        a.energy = r->ering_all + (size_t)i * ECAP_R;
        if (L.has_lin) {
            cpx<float> *lin = reinterpret_cast<cpx<float> *>(base + L.lin);
            kernels_f32().lintab<<<1024, 256, 0, r->stream>>>(lin, run.p.nx, run.p.ny, t.nt, lin_coef(run.p));
            if (cudaGetLastError() != cudaSuccess) return fail(AM_ERR_CUDA);
            a.lintab = lin;
        }
        if (cudaMemcpyAsync(base + L.twx, t.twx.data(), t.twx.size() * sizeof(cpx<float>), cudaMemcpyHostToDevice,
                            r->stream) ||
            cudaMemcpyAsync(base + L.twy, t.twy.data(), t.twy.size() * sizeof(cpx<float>), cudaMemcpyHostToDevice,
                            r->stream) ||
            cudaMemcpyAsync(base + L.kx, t.kx.data(), t.kx.size() * sizeof(float), cudaMemcpyHostToDevice,
                            r->stream) ||
            cudaMemcpyAsync(base + L.ky, t.ky.data(), t.ky.size() * sizeof(float), cudaMemcpyHostToDevice, r->stream))
            return fail(AM_ERR_CUDA);
        // host_setup's tables are per-call locals: finish the copies before they go
        if (cudaStreamSynchronize(r->stream) != cudaSuccess) return fail(AM_ERR_CUDA);
    }
    // Large shared-memory opt-in for every class's kernels.
    const KernelTable<float> &K = kernels_f32();
    const BatchTable &KB = kernels_batch_f32();
    // Work lists (one per pass type) sized for every run at once, full transforms.
    {
        size_t cap = 0;
        for (const RaggedRun &R : r->runs) {
            const int lx = ilog2_exact(R.p.nx), ly = ilog2_exact(R.p.ny);
            const LaunchShape &rs = K.row_shape[lx][0];
            const LaunchShape &cs = K.col_shape[ly][1];
            cap += (size_t)std::max((R.p.ny + rs.per_block - 1) / rs.per_block, col_grid(cs, R.nt, Tile<float>::W));
        }
        r->item_cap = cap;
        if (cudaMalloc(&r->items, 2 * cap * sizeof(WorkItem)) != cudaSuccess) return fail(AM_ERR_OOM);
        const QueueTable &Q = kernels_queue_f32();
        if (Q.row_smem > 48 * 1024 && cudaFuncSetAttribute((const void *)Q.row, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                           (int)Q.row_smem) != cudaSuccess)
            return fail(AM_ERR_CUDA);
        for (int m = 1; m <= 4; m++)
            if (Q.col_smem > 48 * 1024 && cudaFuncSetAttribute((const void *)Q.col[m],
                                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                               (int)Q.col_smem) != cudaSuccess)
                return fail(AM_ERR_CUDA);
    }
    for (const SizeClass &c : r->cls) {
        const size_t rsm = K.row_shape[c.lognx][c.rowv].smem, csm = K.col_shape[c.logny][c.colv].smem;
        if (rsm > 48 * 1024 && cudaFuncSetAttribute((const void *)KB.row[c.lognx][c.rowv],
                                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm))
            return fail(AM_ERR_CUDA);
        for (int m = 0; m < 5; m++)
            if (csm > 48 * 1024 && cudaFuncSetAttribute((const void *)KB.col[c.logny][c.colv][m],
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csm))
                return fail(AM_ERR_CUDA);
        if (csm > 48 * 1024 &&
            cudaFuncSetAttribute((const void *)K.col[c.logny][c.colv][0], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csm))
            return fail(AM_ERR_CUDA);
    }
    *out = r;
    return AM_OK;
}

am_status am_ragged_destroy(am_ragged *r)
{
    if (!r) return AM_OK;
    if (r->stream) cudaStreamSynchronize(r->stream);
    if (r->graph) cudaGraphExecDestroy(r->graph);
    void *ptrs[] = {r->pool, r->stage, r->sc_all, r->ering_all, r->dargs, r->items};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    for (SizeClass &c : r->cls) {
        if (c.branch) cudaStreamDestroy(c.branch);
        if (c.joined) cudaEventDestroy(c.joined);
    }
    if (r->fork) cudaEventDestroy(r->fork);
    if (r->stream) cudaStreamDestroy(r->stream);
    delete r;
    return AM_OK;
}

am_status am_ragged_set_state(am_ragged *r, int run, const void *w_hat, const double mean[2])
{
    if (!r || !w_hat || run < 0 || run >= (int)r->runs.size()) return AM_ERR_ARG;
    RaggedRun &R = r->runs[run];
    const KernelTable<float> &K = kernels_f32();
    const size_t bytes = (size_t)R.p.ny * R.nxh * sizeof(cpx<float>);
    RK(cudaMemcpyAsync(r->stage, w_hat, bytes, cudaMemcpyHostToDevice, r->stream));
    K.tile<<<1024, 256, 0, r->stream>>>(r->stage, R.a.u0, R.p.ny, R.nxh, R.nt, R.p.nx, nullptr);
    RK(cudaGetLastError());
    Scalars s{};
    s.m_new[0] = s.m_old[0] = s.m_appr[0] = mean ? mean[0] : 0.0;
    s.m_new[1] = s.m_old[1] = s.m_appr[1] = mean ? mean[1] : 0.0;
    s.nan_step = -1;
    RK(cudaMemcpyAsync(R.a.sc, &s, sizeof(s), cudaMemcpyHostToDevice, r->stream));
    // start fields with the full transforms (valid however the class is pruned)
    StepArgs<float> a0 = R.a;
    set_pruning<float>(a0, false);
    const SizeClass &C = r->cls[R.cls];
    const LaunchShape &cs = K.col_shape[C.logny][C.colv];
    K.col[C.logny][C.colv][0]<<<col_grid(cs, a0.ntp, Tile<float>::W), cs.threads, cs.smem, r->stream>>>(a0);
    RK(cudaGetLastError());
    RK(cudaStreamSynchronize(r->stream));
    R.inside = state_inside_half_mask<float>((const float *)w_hat, R.p.nx, R.p.ny);
    R.loaded = true;
    R.done = 0;
    if (r->graph) {   // pruning of this run's class may change
        cudaGraphExecDestroy(r->graph);
        r->graph = nullptr;
    }
    return AM_OK;
}

am_status am_ragged_get_state(am_ragged *r, int run, void *w_hat, double mean[2])
{
    if (!r || run < 0 || run >= (int)r->runs.size() || !r->runs[run].loaded) return AM_ERR_ARG;
    const RaggedRun &R = r->runs[run];
    kernels_f32().untile<<<1024, 256, 0, r->stream>>>(R.a.u0, r->stage, R.p.ny, R.nxh, R.nt);
    RK(cudaGetLastError());
    if (w_hat)
        RK(cudaMemcpyAsync(w_hat, r->stage, (size_t)R.p.ny * R.nxh * sizeof(cpx<float>), cudaMemcpyDeviceToHost,
                           r->stream));
    Scalars s;
    RK(cudaMemcpyAsync(&s, R.a.sc, sizeof(s), cudaMemcpyDeviceToHost, r->stream));
    RK(cudaStreamSynchronize(r->stream));
    if (mean) {
        mean[0] = s.m_new[0];
        mean[1] = s.m_new[1];
    }
    return AM_OK;
}

am_status am_ragged_run(am_ragged *r, double *const *energy, int *nan_run, long long *grid_point_steps)
{
    if (nan_run) *nan_run = -1;
    if (grid_point_steps) *grid_point_steps = 0;
    if (!r) return AM_ERR_ARG;
    const int n = (int)r->runs.size();
    for (int i = 0; i < n; i++)
        if (!r->runs[i].loaded) {
            r->err = "run " + std::to_string(i) + " has no state";
            return AM_ERR_ARG;
        }
    std::vector<double> ering((size_t)n * ECAP_R);
    std::vector<Scalars> sc(n);
    long long total = 0;
    for (;;) {
        std::vector<char> act(n, 0);
        long long k = ECAP_R;
        bool any = false;
        for (int i = 0; i < n; i++) {
            const long long left = r->runs[i].nsteps - r->runs[i].done;
            if (left > 0) {
                act[i] = 1;
                any = true;
                k = std::min(k, left);
            }
        }
        if (!any) break;
        am_status st = rebuild(r, act);
        if (st) return st;
        k_ragged_reset_steps<<<(n + 127) / 128, 128, 0, r->stream>>>(r->sc_all, n);
        RK(cudaGetLastError());
        for (long long i = 0; i < k; i++) RK(cudaGraphLaunch(r->graph, r->stream));
        if (energy)
            RK(cudaMemcpy2DAsync(ering.data(), k * sizeof(double), r->ering_all, ECAP_R * sizeof(double),
                                 k * sizeof(double), n, cudaMemcpyDeviceToHost, r->stream));
        RK(cudaMemcpyAsync(sc.data(), r->sc_all, n * sizeof(Scalars), cudaMemcpyDeviceToHost, r->stream));
        RK(cudaStreamSynchronize(r->stream));
        for (int i = 0; i < n; i++) {
            if (!act[i]) continue;
            RaggedRun &R = r->runs[i];
            if (energy && energy[i])
                std::memcpy(energy[i] + R.done, ering.data() + (size_t)i * k, k * sizeof(double));
            if (sc[i].nan_step >= 0) {
                if (nan_run) *nan_run = i;
                r->err = "run " + std::to_string(i) + ": w(0,0) is NaN after step " +
                         std::to_string(R.done + sc[i].nan_step);
                return AM_ERR_NAN;
            }
            R.done += k;
            total += k * (long long)R.p.nx * R.p.ny;
        }
        if (grid_point_steps) *grid_point_steps = total;
    }
    return AM_OK;
}

long long am_ragged_device_bytes(const am_ragged *r)
{
    if (!r) return 0;
    size_t stage = 0;
    for (const RaggedRun &R : r->runs) stage = std::max(stage, (size_t)R.p.ny * R.nxh * sizeof(cpx<float>));
    return (long long)(r->pool_bytes + stage + 2 * r->item_cap * sizeof(WorkItem) +
                       r->runs.size() * (sizeof(Scalars) + ECAP_R * sizeof(double) + sizeof(StepArgs<float>)));
}

int am_ragged_classes(const am_ragged *r) { return r ? (int)r->cls.size() : 0; }

am_status am_ragged_set_mode(am_ragged *r, int mode)
{
    if (!r || (mode != 0 && mode != 1)) return AM_ERR_ARG;
    r->mode = mode;   // the next am_ragged_run rebuilds its graph
    return AM_OK;
}

const char *am_ragged_last_error(const am_ragged *r) { return r ? r->err.c_str() : ""; }

}  // extern "C"
