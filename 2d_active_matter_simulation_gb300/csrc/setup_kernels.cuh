// Set-up kernels: the forward 2-D R2C of a real initial field and the layout
// conversions between the reference's half-plane layout and the tiled layout.
//
// The reference transforms its random initial field with cuFFT R2C, multiplies
// it by the dealias mask and zeroes w(0,0) (ActFlow_V3-2.cu:660-679).  Here the
// same happens in two passes that reuse the step kernels' FFT blocks.
#pragma once
#include "step_kernels.cuh"

namespace af {

// R2C along x of a real field [Ny][Nx] (row-major) into (kx, y) tiled layout.
template <typename T, int LOGNX>
struct RowFwd {
    using RP = RowPass<T, LOGNX>;
    static constexpr int M = RP::M, LOGM = RP::LOGM, R = RP::R, TPC = RP::TPC;
    static constexpr int ROWS = RP::ROWS, THREADS = RP::THREADS, BUFW = RP::BUFW;
    using Buf = typename RP::Buf;
    using FFTf = typename RP::FFTf;
    static constexpr size_t smem_bytes() { return (size_t)ROWS * 2 * BUFW * sizeof(T); }

    template <class Sync>
    static AF_HD void body(const T *src, cpx<T> *dst, const cpx<T> *twx, int ny, int nt, int tid, int bid,
                           unsigned char *smem, Sync &&sync)
    {
        const int rl = tid / TPC, j = tid % TPC;
        const int y = bid * ROWS + rl;
        const bool active = y < ny;
        const int nx = 2 * M;
        T *base = reinterpret_cast<T *>(smem);
        Buf buf{base + (size_t)rl * 2 * BUFW, base + (size_t)rl * 2 * BUFW + BUFW};
        cpx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            int n = j + r * TPC;
            v[r] = active ? mk(src[(size_t)y * nx + 2 * n], src[(size_t)y * nx + 2 * n + 1]) : mk<T>(0, 0);
        }
        FFTf::run(v, j, 0, buf, twx, 2, sync);
        sync();
#pragma unroll
        for (int r = 0; r < R; r++) buf.put(j + r * TPC, 0, v[r]);
        sync();
        const int kend = nt * Tile<T>::W;
        for (int kx = j; kx < kend; kx += TPC) {
            cpx<T> X = mk<T>(0, 0);
            if (kx <= M) {
                cpx<T> A = buf.get(kx & (M - 1), 0);
                cpx<T> B = conj(buf.get((M - kx) & (M - 1), 0));
                cpx<T> E = scale(A + B, (T)0.5);
                cpx<T> D = scale(A - B, (T)0.5);
                X = E + cmul(mk(D.y, -D.x), ldtw(twx, kx));
            }
            if (active) dst[tidx<T>(kx, y, ny)] = X;
        }
    }
};

// Forward FFT along y of a (kx, y) tiled field into (kx, ky); optionally
// multiplied by the dealias mask (dealiasing_func, ActFlow_V3-2.cu:921-932) with
// w(0,0) set to zero (ActFlow_V3-2.cu:679).
template <typename T, int LOGNY>
struct ColFwd {
    using CP = ColPass<T, LOGNY>;
    static constexpr int W = CP::W, R = CP::R, TPC = CP::TPC, TILES = CP::TILES, THREADS = CP::THREADS;
    static constexpr int BUFW = CP::BUFW;
    using Buf = typename CP::Buf;
    using FFTf = typename CP::FFTf;
    static constexpr size_t smem_bytes() { return (size_t)TILES * 2 * BUFW * sizeof(T); }

    template <class Sync>
    static AF_HD void body(const cpx<T> *src, cpx<T> *dst, const cpx<T> *twy, int nx, int ny, int nxh, int nt,
                           int apply_mask, int dealias, int rsq, int tid, int bid, unsigned char *smem, Sync &&sync)
    {
        const int tl = tid / (W * TPC);
        const int rem = tid % (W * TPC);
        const int c = rem % W, j = rem / W;
        const int tile = bid * TILES + tl;
        const bool active = tile < nt;
        const int kx = tile * W + c;
        T *base = reinterpret_cast<T *>(smem);
        Buf buf{base + (size_t)tl * 2 * BUFW, base + (size_t)tl * 2 * BUFW + BUFW};
        const size_t cbase = active ? (size_t)tile * ny * W + c : 0;
        cpx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; r++) v[r] = active ? src[cbase + (size_t)(j + r * TPC) * W] : mk<T>(0, 0);
        FFTf::run(v, j, c, buf, twy, 1, sync);
        if (active) {
#pragma unroll
            for (int r = 0; r < R; r++) {
                int iy = j + r * TPC;
                cpx<T> x = v[r];
                if (kx >= nxh) x = mk<T>(0, 0);
                if (apply_mask) {
                    if (!mask_at(dealias, rsq, nx, ny, kx, iy)) x = mk<T>(0, 0);
                    if (kx == 0 && iy == 0) x = mk<T>(0, 0);
                }
                dst[cbase + (size_t)iy * W] = x;
            }
        }
    }
};

}  // namespace af
