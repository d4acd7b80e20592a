// CPU execution of the CUDA kernel bodies, for the test suite.
//
// The step kernels are written as host/device templates (csrc/fft.cuh,
// csrc/step_kernels.cuh, csrc/setup_kernels.cuh).  This harness compiles them
// with g++ and runs each CTA with one std::thread per CUDA thread and a
// std::barrier for __syncthreads(), using exactly the launch shapes and the
// host set-up (csrc/host_tables.h) of the CUDA build.  It checks the kernels'
// index arithmetic, shared-memory exchange and stage logic against the oracle
// on small grids without a GPU.  It is test code only: the product never runs
// kernels on the CPU.
#include <barrier>
#include <cstring>
#include <functional>
#include <thread>
#include <type_traits>
#include <vector>

#include "host_tables.h"
#include "setup_kernels.cuh"

using namespace af;

namespace {

template <class Body>
void launch(int grid, int threads, size_t smem, Body body)
{
    std::vector<unsigned char> sm(smem, 0);
    for (int b = 0; b < grid; b++) {
        std::barrier bar(threads);
        auto sync = [&bar]() { bar.arrive_and_wait(); };
        std::vector<std::thread> ts;
        ts.reserve(threads);
        for (int t = 0; t < threads; t++) ts.emplace_back([&, t]() { body(t, b, sm.data(), sync); });
        for (auto &th : ts) th.join();
    }
}

template <typename T, int LX, int LY>
struct Runner {
    static int run(const am_params &p, T *w_hat, double *mean, int nsteps, double *energy, int colvar, int rowvar)
    {
        HostTables<T> t;
        StepArgs<T> a{};
        host_setup<T>(p, t, a, 1 << 16);
        // same choice as the C ABI's set_state: pruned transforms under the 1/2
        // rule when the state is zero outside its ellipse
        set_pruning<T>(a, p.dealias == AM_DEALIAS_HALF && state_inside_half_mask<T>(w_hat, p.nx, p.ny));
        const int W = Tile<T>::W, nx = p.nx, ny = p.ny;
        const size_t fsz = (size_t)t.nt * W * ny;
        std::vector<cpx<T>> u0(fsz), acc(fsz), fa(fsz), fx(fsz), fy(fsz), P(fsz), Q(fsz);
        std::vector<double> rowp(side_bytes(ny) / sizeof(double)), en(1 << 16);
        Scalars sc{};
        a.u0 = u0.data(); a.acc = acc.data(); a.fa = fa.data(); a.fx = fx.data(); a.fy = fy.data();
        a.P = P.data(); a.Q = Q.data(); a.twx = t.twx.data(); a.twy = t.twy.data();
        a.kxt = t.kx.data(); a.kyt = t.ky.data(); set_side<T>(a, rowp.data(), ny); a.sc = &sc; a.energy = en.data();
        // integrating-factor table, as the C ABI builds it (k_lintab) when the
        // parameters ask for factors computed in double
        std::vector<cpx<T>> lin;
        if (use_if_table(p)) {
            lin.assign(fsz, mk<T>(0, 0));
            const LinCoef c = lin_coef(p);
            for (int y = 0; y < ny; y++)
                for (int k = 0; k < t.nxh; k++) lin[tidx<T>(k, y, ny)] = lintab_value<T>(c, ny, k, y);
            a.lintab = lin.data();
        }
        // tile the input
        for (int y = 0; y < ny; y++)
            for (int k = 0; k < t.nxh; k++) {
                size_t s = ((size_t)y * t.nxh + k) * 2;
                u0[tidx<T>(k, y, ny)] = mk(w_hat[s], w_hat[s + 1]);
            }
        sc.m_new[0] = mean[0];
        sc.m_new[1] = mean[1];
        sc.nan_step = -1;
        using RP = RowKernel<T, LX>;
        // column-pass launch shape: the build's default for this length, or
        // the radix-8 shape (colvar 2, FP32)
        const int var = colvar == 2 && sizeof(T) == 4 ? 2 : -1;
        auto col = [&](int mode) {
            auto go = [&](auto tag) {
                constexpr int MODE = decltype(tag)::value;
                auto launch_var = [&](auto vtag) {
                    using CP = ColPass<T, LY, MODE, decltype(vtag)::value>;
                    launch(CP::ctas(a), CP::THREADS, CP::smem_bytes(),
                           [&](int tid, int bid, unsigned char *sm, auto &sync) { CP::body(a, tid, bid, sm, sync); });
                };
                // the default shape of the length, and the radix-8 shape at the
                // column lengths its tests use (each instantiation adds to the
                // harness's compile time)
                constexpr int DEF = LY < 11 ? 1 : 0;
                if constexpr (sizeof(T) == 4 && (LY == 7 || LY == 10 || LY == 11)) {
                    if (var == 2) {
                        launch_var(std::integral_constant<int, 2>{});
                        return;
                    }
                }
                launch_var(std::integral_constant<int, DEF>{});
            };
            switch (mode) {
            case 0: go(std::integral_constant<int, 0>{}); break;
            case 1: go(std::integral_constant<int, 1>{}); break;
            case 2: go(std::integral_constant<int, 2>{}); break;
            case 3: go(std::integral_constant<int, 3>{}); break;
            default: go(std::integral_constant<int, 4>{}); break;
            }
        };
        auto row = [&]() {
            if constexpr ((sizeof(T) == 4 || std::is_same_v<T, df>) && LX >= ROWS_LOG_MIN) {
                if (rowvar == 1) {   // row shape with the transforms in sequence (stashes)
                    using RS = RowPassS<T, LX>;
                    launch((ny + RS::ROWS - 1) / RS::ROWS, RS::THREADS, RS::smem_bytes(),
                           [&](int tid, int bid, unsigned char *sm, auto &sync) { RS::body(a, tid, bid, sm, sync); });
                    return;
                }
            }
            launch((ny + RP::ROWS - 1) / RP::ROWS, RP::THREADS, RP::smem_bytes(),
                   [&](int tid, int bid, unsigned char *sm, auto &sync) { RP::body(a, tid, bid, sm, sync); });
        };
        col(0);
        for (int m = 0; m < nsteps; m++) {
            for (int s = 1; s <= 4; s++) {
                row();
                col(s);
            }
        }
        for (int m = 0; m < nsteps; m++) energy[m] = en[m];
        for (int y = 0; y < ny; y++)
            for (int k = 0; k < t.nxh; k++) {
                size_t s = ((size_t)y * t.nxh + k) * 2;
                cpx<T> v = u0[tidx<T>(k, y, ny)];
                w_hat[s] = v.x;
                w_hat[s + 1] = v.y;
            }
        mean[0] = sc.m_new[0];
        mean[1] = sc.m_new[1];
        (void)nx;
        return sc.nan_step;
    }

    static void forward(const am_params &p, const T *real, T *w_hat, int mask)
    {
        HostTables<T> t;
        StepArgs<T> a{};
        host_setup<T>(p, t, a, 16);
        const int W = Tile<T>::W, ny = p.ny;
        const size_t fsz = (size_t)t.nt * W * ny;
        std::vector<cpx<T>> mid(fsz), out(fsz);
        using RF = RowFwd<T, LX>;
        using CF = ColFwd<T, LY>;
        launch((ny + RF::ROWS - 1) / RF::ROWS, RF::THREADS, RF::smem_bytes(),
               [&](int tid, int bid, unsigned char *sm, auto &sync) {
                   RF::body(real, mid.data(), t.twx.data(), ny, t.nt, tid, bid, sm, sync);
               });
        launch((t.nt + CF::TILES - 1) / CF::TILES, CF::THREADS, CF::smem_bytes(),
               [&](int tid, int bid, unsigned char *sm, auto &sync) {
                   CF::body(mid.data(), out.data(), t.twy.data(), p.nx, ny, t.nxh, t.nt, mask, p.dealias,
                            a.rsq, tid, bid, sm, sync);
               });
        for (int y = 0; y < ny; y++)
            for (int k = 0; k < t.nxh; k++) {
                size_t s = ((size_t)y * t.nxh + k) * 2;
                cpx<T> v = out[tidx<T>(k, y, ny)];
                w_hat[s] = v.x;
                w_hat[s + 1] = v.y;
            }
    }
};

// The harness compiles as several translation units in parallel (it is one
// big template instantiation otherwise): with EMU_GROUP = g it instantiates
// the row lengths of group g and exports emu_group_<g>; without it, it holds
// the exported entry points, which call the group of the row length.  Group
// EMU_DF_GROUP holds the double-float kernels (a few grids: 32^2, 64^2, 128x32,
// 2048x8, 8x2048), whose state is exchanged as double.
constexpr int group_of(int lx) { return lx <= 5 ? 0 : lx <= 8 ? 1 : lx <= 10 ? 2 : lx == 11 ? 3 : 4; }
constexpr int NGROUPS = 5;
#define EMU_DF_GROUP 5

struct Call {
    const am_params *p;
    void *w;
    double *m;
    int n;
    double *e;
    const void *real;
    int fwd, mask, colvar, rowvar;
};

#if defined(EMU_GROUP) && EMU_GROUP == EMU_DF_GROUP
template <int LX, int LY>
int run_df(const Call &c)
{
    if (c.fwd) return -100;
    const size_t n = (size_t)c.p->ny * (c.p->nx / 2 + 1) * 2;
    double *wd = (double *)c.w;
    std::vector<df> w(n);
    for (size_t i = 0; i < n; i++) w[i] = df(wd[i]);
    const int r = Runner<df, LX, LY>::run(*c.p, w.data(), c.m, c.n, c.e, c.colvar, c.rowvar);
    for (size_t i = 0; i < n; i++) wd[i] = (double)w[i];
    return r;
}

int dispatch_df(int lx, int ly, const Call &c)
{
    if (lx == 5 && ly == 5) return run_df<5, 5>(c);
    if (lx == 6 && ly == 6) return run_df<6, 6>(c);
    if (lx == 7 && ly == 5) return run_df<7, 5>(c);
    if (lx == 11 && ly == 3) return run_df<11, 3>(c);
    if (lx == 3 && ly == 11) return run_df<3, 11>(c);
    return -100;
}
#elif defined(EMU_GROUP)
template <typename T, int LX, int LY>
int dispatch_y(const Call &c)
{
    T *w = (T *)c.w;
    if (c.fwd) {
        Runner<T, LX, LY>::forward(*c.p, (const T *)c.real, w, c.mask);
        return 0;
    }
    return Runner<T, LX, LY>::run(*c.p, w, c.m, c.n, c.e, c.colvar, c.rowvar);
}

template <typename T, int LX>
int dispatch_x(int ly, const Call &c)
{
    if constexpr (LX <= 7) {
        switch (ly) {
        case 3: return dispatch_y<T, LX, 3>(c);
        case 4: return dispatch_y<T, LX, 4>(c);
        case 5: return dispatch_y<T, LX, 5>(c);
        case 6: return dispatch_y<T, LX, 6>(c);
        case 7: return dispatch_y<T, LX, 7>(c);
        }
        if constexpr (LX <= 4) {   // long columns with few of them: the column kernels at production lengths
            switch (ly) {
            case 9: return dispatch_y<T, LX, 9>(c);
            case 10: return dispatch_y<T, LX, 10>(c);
            case 11: return dispatch_y<T, LX, 11>(c);
            case 12: return dispatch_y<T, LX, 12>(c);
            }
        }
    } else {   // long rows with few of them: the row kernels at production lengths
        switch (ly) {
        case 3: return dispatch_y<T, LX, 3>(c);
        case 4: return dispatch_y<T, LX, 4>(c);
        }
    }
    return -100;
}

template <typename T, int LX>
int dispatch_if_group(int lx, int ly, const Call &c)
{
    if constexpr (group_of(LX) == EMU_GROUP) {
        if (lx == LX) return dispatch_x<T, LX>(ly, c);
    }
    return -200;
}

template <typename T>
int dispatch(int lx, int ly, const Call &c)
{
    int r = -100;
    auto one = [&](int v) {
        if (v != -200) r = v;
    };
    one(dispatch_if_group<T, 3>(lx, ly, c));
    one(dispatch_if_group<T, 4>(lx, ly, c));
    one(dispatch_if_group<T, 5>(lx, ly, c));
    one(dispatch_if_group<T, 6>(lx, ly, c));
    one(dispatch_if_group<T, 7>(lx, ly, c));
    one(dispatch_if_group<T, 9>(lx, ly, c));
    one(dispatch_if_group<T, 10>(lx, ly, c));
    one(dispatch_if_group<T, 11>(lx, ly, c));
    one(dispatch_if_group<T, 12>(lx, ly, c));
    return r;
}
#endif

}  // namespace

#define EMU_CAT2(a, b) a##b
#define EMU_CAT(a, b) EMU_CAT2(a, b)

extern "C" {
#if defined(EMU_GROUP) && EMU_GROUP == EMU_DF_GROUP
int emu_group_df(int lx, int ly, const Call *c) { return dispatch_df(lx, ly, *c); }
#elif defined(EMU_GROUP)
int EMU_CAT(emu_group_, EMU_GROUP)(int lx, int ly, const Call *c)
{
    return c->p->precision == AM_FP64 ? dispatch<double>(lx, ly, *c) : dispatch<float>(lx, ly, *c);
}
#else
int emu_group_0(int, int, const Call *);
int emu_group_1(int, int, const Call *);
int emu_group_2(int, int, const Call *);
int emu_group_3(int, int, const Call *);
int emu_group_4(int, int, const Call *);
int emu_group_df(int, int, const Call *);

static int dispatch_all(const Call &c)
{
    int lx = 0, ly = 0;
    while ((1 << lx) < c.p->nx) lx++;
    while ((1 << ly) < c.p->ny) ly++;
    int (*const groups[NGROUPS])(int, int, const Call *) = {emu_group_0, emu_group_1, emu_group_2, emu_group_3,
                                                            emu_group_4};
    if (c.p->precision == AM_DF64) return emu_group_df(lx, ly, &c);
    return lx < 3 || lx > 12 ? -100 : groups[group_of(lx)](lx, ly, &c);
}

// Advance (w_hat [ny][nx/2+1] complex of the precision, mean[2]) nsteps steps
// with column-pass shape colvar (2: radix 8, FP32, column lengths 128, 1024,
// 2048; otherwise the default for the length) and row-pass shape rowvar (0
// lockstep, 1 in sequence with stashes: FP32 and double-float, Nx >= 1024).
// Returns the first NaN step or -1; -100 for an unsupported size (8..128 each,
// or one side 512..4096 with the other 8..16; double-float, w_hat in double:
// 32x32, 64x64, 128x32, 2048x8, 8x2048).
int emu_run(const am_params *p, void *w_hat, double *mean, int nsteps, double *energy, int colvar, int rowvar)
{
    return dispatch_all(Call{p, w_hat, mean, nsteps, energy, nullptr, 0, 0, colvar, rowvar});
}

// The host check behind pruned transforms (host_tables.h): 1 if the half-plane
// state is zero at every mode the 1/2 rule removes.
int emu_inside_half(const am_params *p, const void *w_hat)
{
    if (p->precision != AM_FP32) return state_inside_half_mask<double>((const double *)w_hat, p->nx, p->ny) ? 1 : 0;
    return state_inside_half_mask<float>((const float *)w_hat, p->nx, p->ny) ? 1 : 0;
}

int emu_forward(const am_params *p, const void *real, void *w_hat, int mask)
{
    return dispatch_all(Call{p, w_hat, nullptr, 0, nullptr, real, 1, mask, -1, 0});
}
#endif
}
