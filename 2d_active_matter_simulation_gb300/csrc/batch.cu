// Ensembles: many simulations of one grid advanced by the same launches.
//
// A batch holds B members with the same grid, box, time step, precision
// (FP32), operator form and dealiasing, and their own lambda, alpha, beta,
// Gamma0, Gamma2, state and mean flow.  Each pass of a step is one launch for
// all members (blockIdx.y = member), the 8 launches of a step are captured once
// in a CUDA graph, so a 64-member ensemble of 512^2 grids costs the GPU 8
// launches per step instead of 512.  Every member computes exactly what a lone
// handle with its parameters computes (the same kernel bodies and arguments).
//
// Device memory per member: the 7 fields of a lone handle, its row sums,
// scalars and energy ring; the twiddle and wavenumber tables and one staging
// buffer are shared.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "actflow.h"
#include "host_tables.h"
#include "kernels.h"

using namespace af;

namespace {
constexpr int ECAP_B = 1024;   // energy ring entries per member
}

struct am_batch {
    std::vector<am_params> p;
    int B = 0, nx = 0, ny = 0, nxh = 0, nt = 0, lognx = 0, logny = 0;
    int colv = 0;                   // column-pass launch shape (0 wide, 1 narrow, 2 wide radix 8)
    int rowv = 0;                   // row-pass launch shape (0 radix 8, 1 radix 16 with stashes)
    cudaStream_t stream = nullptr;
    size_t field_elems = 0;
    cpx<float> *fields = nullptr;   // [B][7][field]
    cpx<float> *lin = nullptr;      // [B][field] integrating-factor tables (members with AM_IF_DOUBLE)
    cpx<float> *stage = nullptr;
    cpx<float> *twx = nullptr, *twy = nullptr;
    float *kxt = nullptr, *kyt = nullptr;
    double *rowp = nullptr, *energy = nullptr;
    Scalars *sc = nullptr;
    StepArgs<float> *dargs = nullptr;
    std::vector<StepArgs<float>> hargs;
    std::vector<char> loaded, inside;
    bool args_dirty = true;
    int ntp_graph = -1;
    cudaGraphExec_t graph = nullptr;
    std::string err;
    // lockstep row shape: its tensor-map form over one map of every member's
    // fields, where the kernel is built and a row's carried tiles fit
    RowTma tma{};
    bool tma_ok = false;
};

#define BK(call)                                                  \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) {                                  \
            b->err = std::string(#call) + ": " + cudaGetErrorString(e_); \
            return e_ == cudaErrorMemoryAllocation ? AM_ERR_OOM : AM_ERR_CUDA; \
        }                                                         \
    } while (0)

namespace {

__global__ void k_batch_reset_steps(Scalars *sc, int B)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < B) sc[i].step = 0;
}

am_status upload_args(am_batch *b)
{
    if (!b->args_dirty) return AM_OK;
    bool pruned = b->p[0].dealias == AM_DEALIAS_HALF;
    for (int i = 0; i < b->B; i++) pruned = pruned && b->inside[i];
    for (auto &a : b->hargs) set_pruning<float>(a, pruned);
    BK(cudaMemcpyAsync(b->dargs, b->hargs.data(), b->B * sizeof(StepArgs<float>), cudaMemcpyHostToDevice, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    b->args_dirty = false;
    return AM_OK;
}

am_status build_graph(am_batch *b)
{
    am_status st = upload_args(b);
    if (st) return st;
    const int ntp = b->hargs[0].ntp;
    if (b->graph && b->ntp_graph == ntp) return AM_OK;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    const KernelTable<float> &K = kernels_f32();
    const BatchTable &KB = kernels_batch_f32();
    // the lockstep row pass fetches its rows by tensor-map copies where the
    // carried tiles fit one exchange buffer (results bit for bit the same)
    b->tma_ok = false;
    if (b->rowv == 0 && KB.row_tma[b->lognx]) {
        const int W = Tile<float>::W;
        const int nbox = (ntp + 255) / 256, box = ((ntp + nbox - 1) / nbox + 3) / 4 * 4;
        if (nbox * box * W <= KB.row_tma_cap[b->lognx] &&
            encode_row_map(&b->tma.map[0], b->fields, b->ny, b->nt, 7 * b->B, b->field_elems * sizeof(cpx<float>),
                           box)) {
            b->tma.nbox = nbox;
            b->tma.box = box;
            b->tma.shared = 1;
            b->tma.slot[0] = 4;   // fy
            b->tma.slot[1] = 3;   // fx
            b->tma.slot[2] = 2;   // fa
            b->tma_ok = true;
        }
    }
    const LaunchShape &rs = b->tma_ok ? KB.row_tma_shape[b->lognx] : K.row_shape[b->lognx][b->rowv];
    const LaunchShape &cs = K.col_shape[b->logny][b->colv];
    const dim3 rgrid((b->ny + rs.per_block - 1) / rs.per_block, b->B);
    const dim3 cgrid(col_grid(cs, ntp, Tile<float>::W), b->B);
    if (b->tma_ok && rs.smem > 48 * 1024)
        BK(cudaFuncSetAttribute((const void *)KB.row_tma[b->lognx], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)rs.smem));
    cudaGraph_t g;
    BK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 1; s <= 4; s++) {
        if (b->tma_ok)
            KB.row_tma[b->lognx]<<<rgrid, rs.threads, rs.smem, b->stream>>>(b->dargs, b->tma);
        else
            KB.row[b->lognx][b->rowv]<<<rgrid, rs.threads, rs.smem, b->stream>>>(b->dargs);
        KB.col[b->logny][b->colv][s]<<<cgrid, cs.threads, cs.smem, b->stream>>>(b->dargs);
    }
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess) {
        b->err = std::string("capture: ") + cudaGetErrorString(e);
        return AM_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->err = std::string("instantiate: ") + cudaGetErrorString(e);
        return AM_ERR_CUDA;
    }
    b->ntp_graph = ntp;
    return AM_OK;
}

}  // namespace

extern "C" {

am_status am_batch_create(const am_params *params, int nmembers, am_batch **out)
{
    if (!params || !out || nmembers < 1) return AM_ERR_ARG;
    *out = nullptr;
    const am_params &p0 = params[0];
    auto lg = [](int n) {
        int l = 0;
        while ((1 << l) < n) l++;
        return (1 << l) == n ? l : -1;
    };
    const int lx = lg(p0.nx), ly = lg(p0.ny);
    if (lx < BATCH_LOG_MIN || lx > BATCH_LOG_MAX || ly < BATCH_LOG_MIN || ly > BATCH_LOG_MAX)
        return AM_ERR_UNSUPPORTED;
    if (p0.precision != AM_FP32) return AM_ERR_UNSUPPORTED;
    for (int i = 1; i < nmembers; i++) {
        const am_params &q = params[i];
        if (q.nx != p0.nx || q.ny != p0.ny || q.lx != p0.lx || q.ly != p0.ly || q.dt != p0.dt ||
            q.precision != p0.precision || q.form != p0.form || q.dealias != p0.dealias)
            return AM_ERR_ARG;
    }
    if (p0.dealias < 0 || p0.dealias > 2 || (p0.form != AM_FORM_REFERENCE && p0.form != AM_FORM_GENERAL))
        return AM_ERR_ARG;
    bool any_lin = false;
    for (int i = 0; i < nmembers; i++) {
        if (params[i].if_factors < AM_IF_AUTO || params[i].if_factors > AM_IF_DOUBLE) return AM_ERR_ARG;
        any_lin = any_lin || use_if_table(params[i]);
    }
    am_batch *b = new (std::nothrow) am_batch();
    if (!b) return AM_ERR_OOM;
    b->p.assign(params, params + nmembers);
    b->B = nmembers;
    b->nx = p0.nx;
    b->ny = p0.ny;
    b->lognx = lx;
    b->logny = ly;
    b->colv = col_variant(AM_FP32, ly);
    b->rowv = row_variant(AM_FP32, lx);
    if (b->rowv == ROWV_TMA) b->rowv = 0;   // single-handle shape; its batched form is the lockstep pass
    b->loaded.assign(nmembers, 0);
    b->inside.assign(nmembers, 0);
    auto fail = [&](am_status s) {
        am_batch_destroy(b);
        return s;
    };
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(AM_ERR_CUDA);
    HostTables<float> t;
    b->hargs.resize(nmembers);
    for (int i = 0; i < nmembers; i++) host_setup<float>(b->p[i], t, b->hargs[i], ECAP_B);
    b->nxh = t.nxh;
    b->nt = t.nt;
    b->field_elems = (size_t)t.nt * Tile<float>::W * b->ny;
    const size_t fbytes = b->field_elems * sizeof(cpx<float>);
    const size_t B = (size_t)nmembers;
    if (cudaMalloc(&b->fields, B * 7 * fbytes) != cudaSuccess) return fail(AM_ERR_OOM);
    if (cudaMemsetAsync(b->fields, 0, B * 7 * fbytes, b->stream) != cudaSuccess) return fail(AM_ERR_CUDA);
    if (any_lin && cudaMalloc(&b->lin, B * fbytes) != cudaSuccess) return fail(AM_ERR_OOM);
    if (cudaMalloc(&b->stage, (size_t)b->ny * b->nxh * sizeof(cpx<float>)) != cudaSuccess ||
        cudaMalloc(&b->twx, b->nx * sizeof(cpx<float>)) != cudaSuccess ||
        cudaMalloc(&b->twy, b->ny * sizeof(cpx<float>)) != cudaSuccess ||
        cudaMalloc(&b->kxt, t.kx.size() * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&b->kyt, t.ky.size() * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&b->rowp, B * side_bytes(b->ny)) != cudaSuccess ||
        cudaMalloc(&b->energy, B * ECAP_B * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&b->sc, B * sizeof(Scalars)) != cudaSuccess ||
        cudaMalloc(&b->dargs, B * sizeof(StepArgs<float>)) != cudaSuccess)
        return fail(AM_ERR_OOM);
    if (cudaMemcpyAsync(b->twx, t.twx.data(), b->nx * sizeof(cpx<float>), cudaMemcpyHostToDevice, b->stream) ||
        cudaMemcpyAsync(b->twy, t.twy.data(), b->ny * sizeof(cpx<float>), cudaMemcpyHostToDevice, b->stream) ||
        cudaMemcpyAsync(b->kxt, t.kx.data(), t.kx.size() * sizeof(float), cudaMemcpyHostToDevice, b->stream) ||
        cudaMemcpyAsync(b->kyt, t.ky.data(), t.ky.size() * sizeof(float), cudaMemcpyHostToDevice, b->stream) ||
        cudaMemsetAsync(b->rowp, 0, B * side_bytes(b->ny), b->stream) ||
        cudaStreamSynchronize(b->stream))
        return fail(AM_ERR_CUDA);
    for (int i = 0; i < nmembers; i++) {
        StepArgs<float> &a = b->hargs[i];
        cpx<float> *f = b->fields + (size_t)i * 7 * b->field_elems;
        a.u0 = f;
        a.acc = f + b->field_elems;
        a.tma_field0 = 7 * i;   // fields [B][7] in one block: the ensemble's shared tensor map
        a.fa = f + 2 * b->field_elems;
        a.fx = f + 3 * b->field_elems;
        a.fy = f + 4 * b->field_elems;
        a.P = f + 5 * b->field_elems;
        a.Q = f + 6 * b->field_elems;
        a.twx = b->twx;
        a.twy = b->twy;
        a.kxt = b->kxt;
        a.kyt = b->kyt;
        set_side<float>(a, reinterpret_cast<unsigned char *>(b->rowp) + i * side_bytes(b->ny), b->ny);
        a.sc = b->sc + i;
        a.energy = b->energy + (size_t)i * ECAP_B;
        if (use_if_table(b->p[i])) {
            cpx<float> *lin = b->lin + (size_t)i * b->field_elems;
            kernels_f32().lintab<<<1024, 256, 0, b->stream>>>(lin, b->nx, b->ny, b->nt, lin_coef(b->p[i]));
            if (cudaGetLastError() != cudaSuccess) return fail(AM_ERR_CUDA);
            a.lintab = lin;
        }
    }
    // Large shared-memory opt-in for the batched kernels (same sizes as the single ones).
    const KernelTable<float> &K = kernels_f32();
    const BatchTable &KB = kernels_batch_f32();
    const size_t rsm = K.row_shape[lx][b->rowv].smem, csm = K.col_shape[ly][b->colv].smem;
    if (rsm > 48 * 1024 && cudaFuncSetAttribute((const void *)KB.row[lx][b->rowv],
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm))
        return fail(AM_ERR_CUDA);
    for (int m = 0; m < 5; m++)
        if (csm > 48 * 1024 &&
            cudaFuncSetAttribute((const void *)KB.col[ly][b->colv][m], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csm))
            return fail(AM_ERR_CUDA);
    // am_batch_set_state starts a member with the single-simulation stage-0 kernel
    if (csm > 48 * 1024 &&
        cudaFuncSetAttribute((const void *)K.col[ly][b->colv][0], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csm))
        return fail(AM_ERR_CUDA);
    *out = b;
    return AM_OK;
}

am_status am_batch_destroy(am_batch *b)
{
    if (!b) return AM_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    void *ptrs[] = {b->fields, b->lin, b->stage, b->twx, b->twy, b->kxt, b->kyt, b->rowp, b->energy, b->sc,
                    b->dargs};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return AM_OK;
}

am_status am_batch_set_state(am_batch *b, int member, const void *w_hat, const double mean[2])
{
    if (!b || !w_hat || member < 0 || member >= b->B) return AM_ERR_ARG;
    const size_t bytes = (size_t)b->ny * b->nxh * sizeof(cpx<float>);
    const KernelTable<float> &K = kernels_f32();
    StepArgs<float> &a = b->hargs[member];
    BK(cudaMemcpyAsync(b->stage, w_hat, bytes, cudaMemcpyHostToDevice, b->stream));
    K.tile<<<1024, 256, 0, b->stream>>>(b->stage, a.u0, b->ny, b->nxh, b->nt, b->nx, nullptr);
    BK(cudaGetLastError());
    Scalars s{};
    s.m_new[0] = s.m_old[0] = s.m_appr[0] = mean ? mean[0] : 0.0;
    s.m_new[1] = s.m_old[1] = s.m_appr[1] = mean ? mean[1] : 0.0;
    s.nan_step = -1;
    BK(cudaMemcpyAsync(a.sc, &s, sizeof(s), cudaMemcpyHostToDevice, b->stream));
    // Start fields of this member with the full transforms (valid whichever
    // way the batch is pruned later).
    StepArgs<float> a0 = a;
    set_pruning<float>(a0, false);
    const LaunchShape &cs = K.col_shape[b->logny][b->colv];
    K.col[b->logny][b->colv][0]<<<col_grid(cs, a0.ntp, Tile<float>::W), cs.threads, cs.smem, b->stream>>>(a0);
    BK(cudaGetLastError());
    BK(cudaStreamSynchronize(b->stream));
    b->inside[member] = state_inside_half_mask<float>((const float *)w_hat, b->nx, b->ny);
    b->loaded[member] = 1;
    b->args_dirty = true;
    return AM_OK;
}

am_status am_batch_get_state(am_batch *b, int member, void *w_hat, double mean[2])
{
    if (!b || member < 0 || member >= b->B || !b->loaded[member]) return AM_ERR_ARG;
    const KernelTable<float> &K = kernels_f32();
    const StepArgs<float> &a = b->hargs[member];
    K.untile<<<1024, 256, 0, b->stream>>>(a.u0, b->stage, b->ny, b->nxh, b->nt);
    BK(cudaGetLastError());
    if (w_hat)
        BK(cudaMemcpyAsync(w_hat, b->stage, (size_t)b->ny * b->nxh * sizeof(cpx<float>), cudaMemcpyDeviceToHost,
                           b->stream));
    Scalars s;
    BK(cudaMemcpyAsync(&s, a.sc, sizeof(s), cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    if (mean) {
        mean[0] = s.m_new[0];
        mean[1] = s.m_new[1];
    }
    return AM_OK;
}

am_status am_batch_step(am_batch *b, int nsteps, double *energy, int *nan_member)
{
    if (nan_member) *nan_member = -1;
    if (!b || nsteps < 0) return AM_ERR_ARG;
    for (int i = 0; i < b->B; i++)
        if (!b->loaded[i]) {
            b->err = "member " + std::to_string(i) + " has no state";
            return AM_ERR_ARG;
        }
    am_status st = build_graph(b);
    if (st) return st;
    std::vector<Scalars> sc(b->B);
    std::vector<double> ering(energy ? (size_t)b->B * ECAP_B : 0);
    int done = 0;
    while (done < nsteps) {
        const int k = nsteps - done < ECAP_B ? nsteps - done : ECAP_B;
        k_batch_reset_steps<<<(b->B + 127) / 128, 128, 0, b->stream>>>(b->sc, b->B);
        BK(cudaGetLastError());
        for (int i = 0; i < k; i++) BK(cudaGraphLaunch(b->graph, b->stream));
        // member rings [B][ECAP_B] -> host [B][k], transposed into the caller's [nsteps][B]
        if (energy)
            BK(cudaMemcpy2DAsync(ering.data(), k * sizeof(double), b->energy, ECAP_B * sizeof(double),
                                 k * sizeof(double), b->B, cudaMemcpyDeviceToHost, b->stream));
        BK(cudaMemcpyAsync(sc.data(), b->sc, b->B * sizeof(Scalars), cudaMemcpyDeviceToHost, b->stream));
        BK(cudaStreamSynchronize(b->stream));
        if (energy)
            for (int m = 0; m < b->B; m++)
                for (int i = 0; i < k; i++) energy[(size_t)(done + i) * b->B + m] = ering[(size_t)m * k + i];
        for (int m = 0; m < b->B; m++)
            if (sc[m].nan_step >= 0) {
                if (nan_member) *nan_member = m;
                b->err = "member " + std::to_string(m) + ": w(0,0) is NaN after step " +
                         std::to_string(done + sc[m].nan_step);
                return AM_ERR_NAN;
            }
        for (int m = 0; m < b->B; m++)
            if (sc[m].status != 0) {
                b->err = "member " + std::to_string(m) + ": a row pass's tensor-map copies did not complete in time";
                return AM_ERR_TIMEOUT;
            }
        done += k;
    }
    return AM_OK;
}

const char *am_batch_last_error(const am_batch *b) { return b ? b->err.c_str() : ""; }

}  // extern "C"
