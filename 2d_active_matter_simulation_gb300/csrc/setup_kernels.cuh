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
    static constexpr int M = RP::M, R = RP::R, TPC = RP::TPC;
    static constexpr int ROWS = RP::ROWS, THREADS = RP::THREADS, BUFS = RP::BUFS;
    using Buf = typename RP::Buf;
    using FFTf = typename RP::FFTf;
    static constexpr size_t smem_bytes() { return RP::smem_bytes(); }

    template <class Sync>
    static AF_HD void body(const T *src, cpx<T> *dst, const cpx<T> *twx, int ny, int nt, int tid, int bid,
                           unsigned char *smem, Sync &&sync)
    {
        const int rl = tid / TPC, j = tid % TPC;
        const int yy = bid * ROWS + rl;
        const bool active = yy < ny;
        const int y = active ? yy : ny - 1;
        const int nx = 2 * M;
        Buf buf{reinterpret_cast<cpx<T> *>(smem) + (size_t)rl * 2 * BUFS};
        cpx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            int n = j + r * TPC;
            v[r] = mk(src[(size_t)y * nx + 2 * n], src[(size_t)y * nx + 2 * n + 1]);
        }
        FFTf::run(v, j, 0, buf, twx, 2, sync);
        sync();
#pragma unroll
        for (int r = 0; r < R; r++) buf.put(j + r * TPC, 0, v[r]);
        sync();
#pragma unroll
        for (int r = 0; r < R; r++) {
            int k = j + r * TPC;
            cpx<T> X = RP::unpack(v[r], buf.get((M - k) & (M - 1), 0), ldtw(twx, k));
            if (active) dst[tidx<T>(k, y, ny)] = X;
        }
        if (active && j == 0) dst[tidx<T>(M, y, ny)] = RP::unpack(v[0], v[0], mk<T>(-1, 0));
        for (int kx = M + 1 + j; active && kx < nt * Tile<T>::W; kx += TPC) dst[tidx<T>(kx, y, ny)] = mk<T>(0, 0);
    }
};

// Forward FFT along y of a (kx, y) tiled field into (kx, ky); optionally
// multiplied by the dealias mask (dealiasing_func, ActFlow_V3-2.cu:921-932) with
// w(0,0) set to zero (ActFlow_V3-2.cu:679).
template <typename T, int LOGNY>
struct ColFwd {
    using CP = ColPass<T, LOGNY, 0>;
    // one tile of W columns per group of W * TPC threads
    static constexpr int W = Tile<T>::W, R = CP::R, TPC = CP::TPC;
    static constexpr int TILES = W * TPC >= 128 ? 1 : 128 / (W * TPC), THREADS = TILES * W * TPC;
    using Buf = XBuf<T, W, 0>;
    static constexpr int BUFS = (Buf::slots(CP::L) + 7) / 8 * 8;
    using FFTf = typename CP::FFTf;
    static constexpr size_t smem_bytes() { return (size_t)TILES * BUFS * sizeof(cpx<T>); }

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
        Buf buf{reinterpret_cast<cpx<T> *>(smem) + (size_t)tl * BUFS};
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
