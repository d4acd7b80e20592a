// am_step_noalloc: the IF-RK4 step without any memory allocation.
//
// Some callers cannot allocate device memory: a plug-in running inside a host
// application that owns the whole device-memory budget (and forbids its plug-ins
// to call cudaMalloc), or a real-time loop that must not take the allocator's
// implicit synchronisation and latency.  For them this entry point runs the same
// step kernels as am_step, with every intermediate buffer (the tiled state,
// stage fields, products, row sums, tables and scalars) carved out of one
// file-scope device array of fixed size.  The caller passes only its inputs and
// outputs, in device memory.
//
// The array is statically sized (kScratchBytes) and every GPU that loads the
// library holds it until the process exits.  All calls share it and it keeps
// the last call's contents, so calls that overlap on the GPU (different streams,
// threads or processes sharing a context) race on it; serialise them.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>

#include "actflow.h"
#include "host_tables.h"
#include "kernels.h"

using namespace af;

namespace {

constexpr size_t kScratchBytes = 8u << 20;   // 8 MiB per device
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Device address of g_scratch per device, looked up once per device with that
// device current (the symbol name is only a host-side stand-in).  The address
// belongs to the device's context: cudaDeviceReset destroys that context and
// the array with it, so the cached address must not be used after a reset
// (the entry point's documentation says so).
constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_ptr[kMaxDevices];

am_status scratch_address(unsigned char **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return AM_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return AM_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return AM_ERR_CUDA;
        g_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_ptr[dev];
    return AM_OK;
}

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

// Twiddle and wavenumber tables, built on the device (no host staging):
// exp(-2 pi i m / N) in double rounded to T; k = 2 pi / L * n in double with L
// held in T, rounded to T.
template <typename T>
__global__ void k_tables(cpx<T> *twx, cpx<T> *twy, T *kx, T *ky, int nx, int ny, int nxh, int nkx, T lx, T ly)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nx) {
        double s, c;
        sincospi(-2.0 * i / nx, &s, &c);
        twx[i] = mk((T)c, (T)s);
    }
    if (i < ny) {
        double s, c;
        sincospi(-2.0 * i / ny, &s, &c);
        twy[i] = mk((T)c, (T)s);
        ky[i] = (T)(2.0 * M_PI / (double)ly * (i < ny / 2 + 1 ? i : i - ny));
    }
    if (i < nkx) kx[i] = i < nxh ? (T)(2.0 * M_PI / (double)lx * i) : (T)0;
}

// Scalars from the caller's mean (init) or back to it.
__global__ void k_mean(Scalars *s, double *mean, int init)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (init) {
        Scalars z{};
        z.m_new[0] = z.m_old[0] = z.m_appr[0] = mean[0];
        z.m_new[1] = z.m_old[1] = z.m_appr[1] = mean[1];
        z.step = 0;
        z.nan_step = -1;
        *s = z;
    } else {
        mean[0] = s->m_new[0];
        mean[1] = s->m_new[1];
    }
}

template <typename T>
const KernelTable<T> &table();
template <>
const KernelTable<float> &table<float>() { return kernels_f32(); }
template <>
const KernelTable<double> &table<double>() { return kernels_f64(); }

template <typename T>
am_status run(const am_params &p, void *w_hat, double *mean, int nsteps, double *energy, cudaStream_t st)
{
    const int nx = p.nx, ny = p.ny, W = Tile<T>::W;
    const int nxh = nx / 2 + 1, nt = (nxh + W - 1) / W, nkx = nt * W;
    int lx2 = 0, ly2 = 0;
    while ((1 << lx2) < nx) lx2++;
    while ((1 << ly2) < ny) ly2++;

    // Carve the scratch: 7 fields, tables, row sums, scalars, a small energy ring.
    const size_t field = align256((size_t)nkx * ny * sizeof(cpx<T>));
    size_t off = 0;
    size_t o_fields = off;
    off += 7 * field;
    size_t o_twx = off;
    off += align256((size_t)nx * sizeof(cpx<T>));
    size_t o_twy = off;
    off += align256((size_t)ny * sizeof(cpx<T>));
    size_t o_kx = off;
    off += align256((size_t)nkx * sizeof(T));
    size_t o_ky = off;
    off += align256((size_t)ny * sizeof(T));
    size_t o_rowp = off;
    off += align256(side_bytes(ny));
    size_t o_sc = off;
    off += align256(sizeof(Scalars));
    size_t o_ring = off;
    off += align256(16 * sizeof(double));
    if (off > kScratchBytes) return AM_ERR_UNSUPPORTED;

    unsigned char *base = nullptr;
    am_status s = scratch_address(&base);
    if (s) return s;

    StepArgs<T> a{};
    a.nx = nx;
    a.ny = ny;
    a.nxh = nxh;
    a.nt = nt;
    a.kxp = nxh - 1;   // full transforms
    a.ntp = nt;
    cpx<T> *f = reinterpret_cast<cpx<T> *>(base + o_fields);
    const size_t fe = field / sizeof(cpx<T>);
    a.u0 = f;
    a.acc = f + fe;
    a.fa = f + 2 * fe;
    a.fx = f + 3 * fe;
    a.fy = f + 4 * fe;
    a.P = f + 5 * fe;
    a.Q = f + 6 * fe;
    a.twx = reinterpret_cast<const cpx<T> *>(base + o_twx);
    a.twy = reinterpret_cast<const cpx<T> *>(base + o_twy);
    a.kxt = reinterpret_cast<const T *>(base + o_kx);
    a.kyt = reinterpret_cast<const T *>(base + o_ky);
    set_side<T>(a, base + o_rowp, ny);
    a.sc = reinterpret_cast<Scalars *>(base + o_sc);
    a.energy = energy ? energy : reinterpret_cast<double *>(base + o_ring);
    a.ecap = energy ? (nsteps > 0 ? nsteps : 1) : 16;
    // Physics scalars, the same formulas as the handle path (host_tables.h):
    // lambda / N^2 and beta / N^3 in T, mean-flow factors in double.
    const T fnorm = (T)(nx * ny);
    a.lam_s = (T)p.lambda / (fnorm * fnorm);
    a.beta_s = (T)p.beta / (fnorm * fnorm * fnorm);
    const double nd = (double)nx * (double)ny;
    a.beta_sd = p.beta / (nd * nd * nd);
    a.dt = (T)p.dt;
    a.alpha = (T)p.alpha;
    a.g0 = (T)p.gamma0;
    a.g2 = (T)p.gamma2;
    a.form = p.form;
    a.dealias = p.dealias;
    a.rsq = reference_rsq(nx, ny);
    const double L0 = p.form == AM_FORM_REFERENCE ? -(1.0 + p.alpha) : -p.alpha;
    a.lin_v = std::exp(L0 * p.dt);
    a.lin2_v = std::exp(L0 * p.dt / 2);
    set_mean_flow_coeffs<T>(a);
    a.inv_2n3 = 1.0 / (2.0 * nd * nd * nd);

    const KernelTable<T> &K = table<T>();
    constexpr int prec = sizeof(T) == 8 ? AM_FP64 : AM_FP32;
    const int rowv = row_variant(prec, lx2) == ROWV_TMA ? 0 : row_variant(prec, lx2);   // no tensor maps here
    const LaunchShape &rs = K.row_shape[lx2][rowv];
    const int colv = col_variant(prec, ly2);
    const LaunchShape &cs = K.col_shape[ly2][colv];
    if (rs.smem > 48 * 1024 &&
        cudaFuncSetAttribute((const void *)K.row[lx2][rowv], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rs.smem))
        return AM_ERR_CUDA;
    for (int m = 0; m < 5; m++)
        if (cs.smem > 48 * 1024 && cudaFuncSetAttribute((const void *)K.col[ly2][colv][m],
                                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cs.smem))
            return AM_ERR_CUDA;

    const int nmax = nx > ny ? (nx > nkx ? nx : nkx) : (ny > nkx ? ny : nkx);
    k_tables<T><<<(nmax + 255) / 256, 256, 0, st>>>((cpx<T> *)a.twx, (cpx<T> *)a.twy, (T *)a.kxt, (T *)a.kyt, nx, ny,
                                                   nxh, nkx, (T)p.lx, (T)p.ly);
    k_mean<<<1, 1, 0, st>>>(a.sc, mean, 1);
    K.tile<<<1024, 256, 0, st>>>((const cpx<T> *)w_hat, a.u0, ny, nxh, nt, nx, nullptr);
    const int rgrid = (ny + rs.per_block - 1) / rs.per_block;
    const int cgrid = col_grid(cs, nt, Tile<T>::W);
    StepArgs<T> b = a;
    b.mode = 0;
    K.col[ly2][colv][0]<<<cgrid, cs.threads, cs.smem, st>>>(b);
    for (int n = 0; n < nsteps; n++) {
        for (int stage = 1; stage <= 4; stage++) {
            K.row[lx2][rowv]<<<rgrid, rs.threads, rs.smem, st>>>(a);
            b.mode = stage;
            K.col[ly2][colv][stage]<<<cgrid, cs.threads, cs.smem, st>>>(b);
        }
    }
    K.untile<<<1024, 256, 0, st>>>(a.u0, (cpx<T> *)w_hat, ny, nxh, nt);
    k_mean<<<1, 1, 0, st>>>(a.sc, mean, 0);
    return cudaGetLastError() == cudaSuccess ? AM_OK : AM_ERR_CUDA;
}

}  // namespace

extern "C" am_status am_step_noalloc(const am_params *p, void *w_hat, double *mean, int nsteps, double *energy,
                                     void *stream)
{
    if (!p || !w_hat || !mean || nsteps < 0) return AM_ERR_ARG;
    auto pow2 = [](int n) { return n > 0 && (n & (n - 1)) == 0; };
    if (!pow2(p->nx) || !pow2(p->ny) || p->nx < (1 << LOG_MIN) || p->ny < (1 << LOG_MIN) ||
        p->nx > (1 << LOG_MAX) || p->ny > (1 << LOG_MAX))
        return AM_ERR_UNSUPPORTED;
    if (p->precision == AM_DF64) return AM_ERR_UNSUPPORTED;   // double-float: handles only
    if (p->precision != AM_FP32 && p->precision != AM_FP64) return AM_ERR_ARG;
    if (p->dealias < 0 || p->dealias > 2 || (p->form != AM_FORM_REFERENCE && p->form != AM_FORM_GENERAL))
        return AM_ERR_ARG;
    // the parameter checks of am_create: a non-positive box length makes the
    // wavenumber tables infinite and the state NaN
    if (!(p->lx > 0) || !(p->ly > 0) || !std::isfinite(p->dt)) return AM_ERR_ARG;
    if (p->if_factors < AM_IF_AUTO || p->if_factors > AM_IF_DOUBLE) return AM_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return p->precision == AM_FP64 ? run<double>(*p, w_hat, mean, nsteps, energy, st)
                                   : run<float>(*p, w_hat, mean, nsteps, energy, st);
}
