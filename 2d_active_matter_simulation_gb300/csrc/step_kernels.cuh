// The two fused passes of one integrating-factor RK4 stage.
//
// Reference: ActFlow_V3-2.cu (DominikSuchla/2D_active_matter_simulation).  The
// reference spends a stage on 7 cuFFT 2-D transforms and 5 pointwise kernels
// (nonl_func ActFlow_V3-2.cu:1036-1088, integrate_func_* 940-1018,
// reality_func 1228-1243).  Here a stage is two kernels:
//
//   row pass  (one CTA row group per y):   C2R along x of a, ux, uy ->
//             real-space products P = lam' w ux + beta' |u|^2 uy,
//             Q = lam' w uy - beta' |u|^2 ux and the per-row sums of |u|^2
//             (energy) and |u|^2 u (mean-flow right-hand side) -> R2C along x
//             of P and Q.
//   column pass (one CTA per tile of kx columns): forward FFT along y of P, Q
//             -> N = i (-kx P^ - ky Q^) * mask -> Hermitian repair of the
//             kx = 0 column of the accumulator -> RK stage combination with the
//             integrating factors -> mean-flow scalar update -> Biot-Savart ->
//             inverse FFT along y of the next stage input a, ux, uy.
//
// By linearity F[lam' w ux] + F[beta' |u|^2 uy] = F[P], so the reference's four
// forward transforms of separate products (ActFlow_V3-2.cu:1069-1072) collapse
// into two, and N = i(-kx(lam'A + beta'D) - ky(lam'B - beta'C)) of
// nonl_subfunc_2 (ActFlow_V3-2.cu:1219-1224) becomes i(-kx P^ - ky Q^).
//
// HBM layout ("tiled"): every half-plane field, in (kx, y) or (kx, ky) space,
// is stored as tiles of W adjacent kx columns (W * sizeof(cpx<T>) = 32 bytes, one
// DRAM sector); inside a tile the W values of one row are contiguous and rows
// follow each other:  index(kx, y) = ((kx / W) * Ny + y) * W + kx % W.  The row
// pass reads and writes whole 32-byte sectors per row; the column pass reads and
// writes each tile as one contiguous block.  Tiles past Nx/2 are padding and
// stay zero.
#pragma once
#include "fft.cuh"

namespace af {

struct Scalars {
    double m_old[2], m_new[2], m_appr[2];  // scaled mean velocity Nx*Ny*<u>
    int step;                              // steps completed since set_state
    int nan_step;                          // first step whose w(0,0) is NaN, or -1
    int status;                            // reserved device status word (0 = ok)
    int pad_;
};

template <typename T>
struct StepArgs {
    int nx, ny, nxh, nt;            // grid; nt = number of column tiles
    cpx<T> *u0, *acc;               // spectral state (kx, ky): w_old / w_new
    cpx<T> *fa, *fx, *fy;           // stage input a, ux, uy in (kx, y)
    cpx<T> *P, *Q;                  // products in (kx, y)
    const cpx<T> *twx;              // exp(-2 pi i m / Nx), m < Nx
    const cpx<T> *twy;              // exp(-2 pi i m / Ny), m < Ny
    const T *kxt;                   // kx wavenumbers, nt * W entries (0 past Nx/2)
    const T *kyt;                   // ky wavenumbers in FFT order, Ny entries
    double *rowp;                   // per-row sums [Ny][3]: |u|^2, |u|^2 ux, |u|^2 uy
    Scalars *sc;
    double *energy;                 // energy per step, ring of ecap entries
    int ecap;
    T lam_s, beta_s;                // lambda / N^2, beta / N^3 (FFT normalisation folded in)
    double beta_sd;                 // beta / N^3 in double for the mean-flow update
    T dt, alpha, g0, g2;
    int form;                       // 0: -(1-k^2)^2 - alpha, 1: -alpha - g0 k^2 - g2 k^4
    int dealias;                    // 0: reference (int32 radius), 1: 1/2 rule, 2: none
    int rsq;                        // reference mask radius^2 after 32-bit wrap
    double lin_v, lin2_v;           // mean-flow integrating factors
    double inv_2n3;                 // 1 / (2 N^3)
    int mode;                       // column pass: 0 = start from u0, 1..4 = RK stage
};

// Tile width in columns: 32 bytes of complex values.
template <typename T>
struct Tile {
    static constexpr int W = 32 / (int)sizeof(cpx<T>);
};

template <typename T>
AF_HD size_t tidx(int kx, int y, int ny)
{
    constexpr int W = Tile<T>::W;
    return ((size_t)(kx / W) * ny + y) * W + (kx % W);
}

// Dealiasing mask at half-plane index (ix, iy).  Mode 0 restates cutoff_func
// (ActFlow_V3-2.cu:899-919) with the radius already wrapped to 32 bits on the
// host; mode 1 is the isotropic 1/2 rule; mode 2 keeps every mode.
AF_HD int mask_at(int dealias, int rsq, int nx, int ny, int ix, int iy)
{
    if (dealias == 0) {
        int a = ix * ix + iy * iy;
        int b = ix * ix + (ny - iy) * (ny - iy);
        return (a <= rsq || b <= rsq) ? 1 : 0;
    }
    if (dealias == 1) {
        long long ky = iy <= ny / 2 ? iy : iy - ny;
        long long X = ix, NX = nx, NY = ny;
        return 16 * (X * X * NY * NY + ky * ky * NX * NX) <= NX * NX * NY * NY ? 1 : 0;
    }
    return 1;
}

AF_HD float expT(float x) { return expf(x); }
AF_HD double expT(double x) { return exp(x); }

// ------------------------------------------------------------------ row pass
// Launch: blockDim = ROWS * TPC, gridDim = ceil(Ny / ROWS).
template <typename T, int LOGNX>
struct RowPass {
    static constexpr int M = 1 << (LOGNX - 1);   // complex length of the half-size FFT
    static constexpr int LOGM = LOGNX - 1;
    static constexpr int LOGR = sizeof(T) == 4 ? 3 : 3;
    using FFTi = BlockFFT<T, LOGM, LOGR, +1>;
    using FFTf = BlockFFT<T, LOGM, LOGR, -1>;
    static constexpr int R = FFTi::R;
    static constexpr int TPC = FFTi::TPC;
    static constexpr int ROWS = TPC >= 256 ? 1 : 256 / TPC;
    static constexpr int THREADS = ROWS * TPC;
    using Buf = XBuf<T, 1, 4>;
    static constexpr int BUFW = (Buf::words(M + 1) + 31) / 32 * 32;   // words per row buffer

    static constexpr size_t smem_bytes()
    {
        return (size_t)ROWS * 2 * BUFW * sizeof(T) + (size_t)ROWS * TPC * 3 * sizeof(double);
    }

    template <class Sync>
    static AF_HD void body(const StepArgs<T> &a, int tid, int bid, unsigned char *smem, Sync &&sync)
    {
        const int rl = tid / TPC, j = tid % TPC;
        const int y = bid * ROWS + rl;
        const bool active = y < a.ny;
        const int ny = a.ny;
        T *base = reinterpret_cast<T *>(smem);
        Buf buf{base + (size_t)rl * 2 * BUFW, base + (size_t)rl * 2 * BUFW + BUFW};
        double *red = reinterpret_cast<double *>(base + (size_t)ROWS * 2 * BUFW) + (size_t)rl * TPC * 3;

        cpx<T> z[3][R];
        const cpx<T> *src[3] = {a.fx, a.fy, a.fa};
#pragma unroll
        for (int f = 0; f < 3; f++) {
            sync();
            // Stage X(kx, y), kx = 0..M; the imaginary parts at kx = 0 and kx = M
            // are dropped, as a half-plane C2R does.
            for (int kx = j; kx <= M; kx += TPC) {
                cpx<T> v = mk<T>(0, 0);
                if (active) v = src[f][tidx<T>(kx, y, ny)];
                if (kx == 0 || kx == M) v.y = 0;
                buf.put(kx, 0, v);
            }
            sync();
            // Pack the Hermitian half spectrum into a length-M complex spectrum:
            // Z(k) = E(k) + i O(k), E = X(k) + conj X(M-k),
            // O = (X(k) - conj X(M-k)) * exp(+2 pi i k / Nx).
            cpx<T> v[R];
#pragma unroll
            for (int r = 0; r < R; r++) {
                int k = j + r * TPC;
                cpx<T> A = buf.get(k, 0);
                cpx<T> B = conj(buf.get(M - k, 0));
                cpx<T> E = A + B;
                cpx<T> O = cmulc(A - B, ldtw(a.twx, k));
                v[r] = mk(E.x - O.y, E.y + O.x);
            }
            FFTi::run(v, j, 0, buf, a.twx, 2, sync);
#pragma unroll
            for (int r = 0; r < R; r++) z[f][r] = v[r];
        }

        // Real-space products and per-thread partial sums.  z[.][r] holds the
        // real values at x = 2n (real part) and x = 2n + 1 (imaginary part),
        // n = j + r * TPC.  Order: 0 = ux, 1 = uy, 2 = w.
        T se = 0, sx = 0, sy = 0;
        cpx<T> p[R], q[R];
        const T lam = a.lam_s, bet = a.beta_s;
#pragma unroll
        for (int r = 0; r < R; r++) {
            T ux0 = z[0][r].x, uy0 = z[1][r].x, w0 = z[2][r].x;
            T ux1 = z[0][r].y, uy1 = z[1][r].y, w1 = z[2][r].y;
            T s0 = ux0 * ux0 + uy0 * uy0, s1 = ux1 * ux1 + uy1 * uy1;
            se += s0 + s1;
            sx += s0 * ux0 + s1 * ux1;
            sy += s0 * uy0 + s1 * uy1;
            p[r] = mk(lam * w0 * ux0 + bet * s0 * uy0, lam * w1 * ux1 + bet * s1 * uy1);
            q[r] = mk(lam * w0 * uy0 - bet * s0 * ux0, lam * w1 * uy1 - bet * s1 * ux1);
        }

        // Row sums: tree reduction in double over the TPC threads of the row.
        sync();
        red[j] = (double)se;
        red[TPC + j] = (double)sx;
        red[2 * TPC + j] = (double)sy;
        sync();
        for (int s = TPC / 2; s > 0; s >>= 1) {
            if (j < s) {
                red[j] += red[j + s];
                red[TPC + j] += red[TPC + j + s];
                red[2 * TPC + j] += red[2 * TPC + j + s];
            }
            sync();
        }
        if (active && j == 0) {
            a.rowp[(size_t)y * 3 + 0] = red[0];
            a.rowp[(size_t)y * 3 + 1] = red[TPC];
            a.rowp[(size_t)y * 3 + 2] = red[2 * TPC];
        }

        // Forward R2C along x of P and Q.
#pragma unroll
        for (int f = 0; f < 2; f++) {
            cpx<T> v[R];
#pragma unroll
            for (int r = 0; r < R; r++) v[r] = f == 0 ? p[r] : q[r];
            FFTf::run(v, j, 0, buf, a.twx, 2, sync);
            sync();
#pragma unroll
            for (int r = 0; r < R; r++) buf.put(j + r * TPC, 0, v[r]);
            sync();
            // Unpack: X(k) = E(k) + exp(-2 pi i k / Nx) O(k) with
            // E = (Z(k) + conj Z(M-k)) / 2, O = (Z(k) - conj Z(M-k)) / (2i).
            cpx<T> *dst = f == 0 ? a.P : a.Q;
            const int kend = a.nt * Tile<T>::W;
            for (int kx = j; kx < kend; kx += TPC) {
                cpx<T> X = mk<T>(0, 0);
                if (kx <= M) {
                    cpx<T> A = buf.get(kx & (M - 1), 0);
                    cpx<T> B = conj(buf.get((M - kx) & (M - 1), 0));
                    cpx<T> E = scale(A + B, (T)0.5);
                    cpx<T> D = scale(A - B, (T)0.5);
                    cpx<T> O = mk(D.y, -D.x);
                    X = E + cmul(O, ldtw(a.twx, kx));
                }
                if (active) dst[tidx<T>(kx, y, ny)] = X;
            }
        }
    }
};

// --------------------------------------------------------------- column pass
// Launch: blockDim = TILES * W * TPC, gridDim = ceil(nt / TILES).
template <typename T, int LOGNY>
struct ColPass {
    static constexpr int W = Tile<T>::W;
    static constexpr int LOGR = sizeof(T) == 4 ? 4 : 3;
    using FFTf = BlockFFT<T, LOGNY, LOGR, -1>;
    using FFTi = BlockFFT<T, LOGNY, LOGR, +1>;
    static constexpr int R = FFTf::R;
    static constexpr int TPC = FFTf::TPC;
    static constexpr int L = 1 << LOGNY;
    static constexpr int TILES = W * TPC >= 128 ? 1 : 128 / (W * TPC);
    static constexpr int THREADS = TILES * W * TPC;
    static constexpr int PADK = sizeof(T) == 4 ? 36 : 4;
    using Buf = XBuf<T, W, PADK>;
    static constexpr int BUFW = (Buf::words(L) + 31) / 32 * 32;

    static constexpr size_t smem_bytes()
    {
        return (size_t)TILES * 2 * BUFW * sizeof(T) + (size_t)THREADS * 3 * sizeof(double) + 8 * sizeof(double);
    }

    template <class Sync>
    static AF_HD void body(const StepArgs<T> &a, int tid, int bid, unsigned char *smem, Sync &&sync)
    {
        const int tl = tid / (W * TPC);
        const int rem = tid % (W * TPC);
        const int c = rem % W, j = rem / W;
        const int tile = bid * TILES + tl;
        const bool active = tile < a.nt;
        const int kx = tile * W + c;
        const bool col = active && kx < a.nxh;   // a real (non-padding) column
        const int ny = a.ny, nx = a.nx;
        const int mode = a.mode;
        T *base = reinterpret_cast<T *>(smem);
        Buf buf{base + (size_t)tl * 2 * BUFW, base + (size_t)tl * 2 * BUFW + BUFW};
        double *red = reinterpret_cast<double *>(base + (size_t)TILES * 2 * BUFW);
        double *bc = red + (size_t)THREADS * 3;   // broadcast slots
        const bool owner = bid == 0;              // this CTA holds column kx = 0
        const T kxv = active ? a.kxt[kx] : (T)0;
        const size_t cbase = active ? (size_t)tile * ny * W + c : 0;

        // ---- forward FFT along y of P and Q, assembly of N = i(-kx P^ - ky Q^) * mask
        cpx<T> nl[R];
        if (mode != 0) {
            cpx<T> ph[R], v[R];
#pragma unroll
            for (int r = 0; r < R; r++) v[r] = active ? a.P[cbase + (size_t)(j + r * TPC) * W] : mk<T>(0, 0);
            FFTf::run(v, j, c, buf, a.twy, 1, sync);
#pragma unroll
            for (int r = 0; r < R; r++) ph[r] = v[r];
#pragma unroll
            for (int r = 0; r < R; r++) v[r] = active ? a.Q[cbase + (size_t)(j + r * TPC) * W] : mk<T>(0, 0);
            FFTf::run(v, j, c, buf, a.twy, 1, sync);
#pragma unroll
            for (int r = 0; r < R; r++) {
                int iy = j + r * TPC;
                T kyv = a.kyt[iy];
                T tr = -kxv * ph[r].x - kyv * v[r].x;
                T ti = -kxv * ph[r].y - kyv * v[r].y;
                T m = (col && mask_at(a.dealias, a.rsq, nx, ny, kx, iy)) ? (T)1 : (T)0;
                nl[r] = mk(-ti * m, tr * m);
            }
        }

        // ---- mean flow and energy: reduce the row sums (CTA holding kx = 0)
        if (owner) {
            double se = 0, sx = 0, sy = 0;
            if (mode != 0) {
                for (int y = tid; y < ny; y += THREADS) {
                    se += a.rowp[(size_t)y * 3 + 0];
                    sx += a.rowp[(size_t)y * 3 + 1];
                    sy += a.rowp[(size_t)y * 3 + 2];
                }
            }
            sync();
            red[tid] = se;
            red[THREADS + tid] = sx;
            red[2 * THREADS + tid] = sy;
            sync();
            if (tid == 0) {
                Scalars *s = a.sc;
                double Se = 0, Sx = 0, Sy = 0;
                for (int t = 0; t < THREADS; t++) {
                    Se += red[t];
                    Sx += red[THREADS + t];
                    Sy += red[2 * THREADS + t];
                }
                // Mean-flow right-hand side -beta' Re F[|u|^2 u](0)
                // (ActFlow_V3-2.cu:1086-1087) and its stage updates
                // (ActFlow_V3-2.cu:729-732, 756-759, 778-781, 799-802, 820-821).
                double n0 = -a.beta_sd * Sx, n1 = -a.beta_sd * Sy;
                const double dt = (double)a.dt;
                if (mode == 0) {
                    for (int d = 0; d < 2; d++) {
                        s->m_old[d] = s->m_new[d];
                        s->m_appr[d] = s->m_new[d];
                    }
                } else if (mode == 1) {
                    a.energy[s->step % a.ecap] = Se * a.inv_2n3;
                    s->m_new[0] += dt / 6 * a.lin_v * n0;
                    s->m_new[1] += dt / 6 * a.lin_v * n1;
                    s->m_appr[0] = a.lin2_v * (s->m_old[0] + dt / 2 * n0);
                    s->m_appr[1] = a.lin2_v * (s->m_old[1] + dt / 2 * n1);
                } else if (mode == 2) {
                    s->m_new[0] += dt / 3 * a.lin2_v * n0;
                    s->m_new[1] += dt / 3 * a.lin2_v * n1;
                    s->m_appr[0] = a.lin2_v * (s->m_old[0] + dt / 2 * n0);
                    s->m_appr[1] = a.lin2_v * (s->m_old[1] + dt / 2 * n1);
                } else if (mode == 3) {
                    s->m_new[0] += dt / 3 * a.lin2_v * n0;
                    s->m_new[1] += dt / 3 * a.lin2_v * n1;
                    s->m_appr[0] = a.lin_v * (s->m_old[0] + dt * n0);
                    s->m_appr[1] = a.lin_v * (s->m_old[1] + dt * n1);
                } else {
                    s->m_new[0] += dt / 6 * n0;
                    s->m_new[1] += dt / 6 * n1;
                    for (int d = 0; d < 2; d++) {
                        s->m_old[d] = s->m_new[d];
                        s->m_appr[d] = s->m_new[d];
                    }
                }
                bc[0] = s->m_appr[0];
                bc[1] = s->m_appr[1];
            }
        }

        // ---- RK stage combination (integrate_func_0..4, ActFlow_V3-2.cu:940-1018)
        // with the Hermitian repair of the accumulator's kx = 0 column before
        // the addition (reality_func, ActFlow_V3-2.cu:1228-1243).
        cpx<T> av[R];
        {
            cpx<T> accv[R];
            T E[R], E2[R];
            const T dt = a.dt;
#pragma unroll
            for (int r = 0; r < R; r++) {
                int iy = j + r * TPC;
                T kyv = a.kyt[iy];
                T k2 = kyv * kyv + kxv * kxv;
                T Lk = a.form == 0 ? -(1 - k2) * (1 - k2) - a.alpha : -a.alpha - a.g0 * k2 - a.g2 * k2 * k2;
                E[r] = expT(Lk * dt);
                E2[r] = expT(Lk * dt / 2);
                size_t g = cbase + (size_t)iy * W;
                if (mode == 0) {
                    av[r] = active ? a.u0[g] : mk<T>(0, 0);
                } else if (mode == 1) {
                    cpx<T> u = active ? a.u0[g] : mk<T>(0, 0);
                    av[r] = u;                      // keep u0 for the stage input
                    accv[r] = scale(u, E[r]);       // w_new = w_old * lin
                } else {
                    accv[r] = active ? a.acc[g] : mk<T>(0, 0);
                }
            }
            if (mode != 0) {
                if (owner) {
                    sync();
                    if (tl == 0 && c == 0) {
#pragma unroll
                        for (int r = 0; r < R; r++) buf.put(j + r * TPC, 0, accv[r]);
                    }
                    sync();
                    if (tl == 0 && c == 0) {
#pragma unroll
                        for (int r = 0; r < R; r++) {
                            int iy = j + r * TPC;
                            if (iy >= 1 && iy < ny / 2) {
                                cpx<T> b = buf.get(ny - iy, 0);
                                accv[r] = mk((T)0.5f * (accv[r].x + b.x), (T)0.5f * (accv[r].y - b.y));
                            } else if (iy > ny / 2) {
                                cpx<T> b = buf.get(ny - iy, 0);
                                cpx<T> m = mk((T)0.5f * (b.x + accv[r].x), (T)0.5f * (b.y - accv[r].y));
                                accv[r] = conj(m);
                            }
                        }
                    }
                }
                if (mode != 1) {
#pragma unroll
                    for (int r = 0; r < R; r++) av[r] = active ? a.u0[cbase + (size_t)(j + r * TPC) * W] : mk<T>(0, 0);
                }
#pragma unroll
                for (int r = 0; r < R; r++) {
                    cpx<T> n = nl[r], o = av[r], w = accv[r];
                    size_t g = cbase + (size_t)(j + r * TPC) * W;
                    if (mode == 1) {
                        T f = dt / 6 * E[r];
                        w = mk(w.x + f * n.x, w.y + f * n.y);
                        av[r] = scale(mk(o.x + dt / 2 * n.x, o.y + dt / 2 * n.y), E2[r]);
                    } else if (mode == 2) {
                        T f = dt / 3 * E2[r];
                        w = mk(w.x + f * n.x, w.y + f * n.y);
                        av[r] = scale(mk(o.x + dt / 2 * n.x, o.y + dt / 2 * n.y), E2[r]);
                    } else if (mode == 3) {
                        T f = dt / 3 * E2[r];
                        w = mk(w.x + f * n.x, w.y + f * n.y);
                        av[r] = scale(mk(o.x + dt * n.x, o.y + dt * n.y), E[r]);
                    } else {
                        w = mk(w.x + dt / 6 * n.x, w.y + dt / 6 * n.y);
                        av[r] = w;                  // next step: w_old = w_appr = w_new
                    }
                    if (active) {
                        if (mode == 4) a.u0[g] = w;
                        else a.acc[g] = w;
                    }
                }
                if (mode == 4 && owner && tid == 0) {
                    // NaN probe on Re w(0,0) (check_func, ActFlow_V3-2.cu:884-897).
                    Scalars *s = a.sc;
                    if (av[0].x != av[0].x && s->nan_step < 0) s->nan_step = s->step;
                    s->step += 1;
                }
            }
        }

        // ---- Biot-Savart (nonl_subfunc_0, ActFlow_V3-2.cu:1176-1180) and the
        // mean velocity in the k = 0 slot (ActFlow_V3-2.cu:1053-1054), then the
        // inverse FFT along y of a, ux, uy.
        if (owner) sync();   // bc[] written by thread 0 above
        T m0 = 0, m1 = 0;
        if (owner) {
            m0 = (T)bc[0];
            m1 = (T)bc[1];
        }
#pragma unroll
        for (int f = 0; f < 3; f++) {
            cpx<T> v[R];
#pragma unroll
            for (int r = 0; r < R; r++) {
                int iy = j + r * TPC;
                cpx<T> w = av[r];
                if (f == 0) {
                    v[r] = col ? w : mk<T>(0, 0);
                } else {
                    T kyv = a.kyt[iy];
                    T k2 = kyv * kyv + kxv * kxv;
                    T kk = f == 1 ? kyv : -kxv;
                    cpx<T> iw = mk(-w.y, w.x);
                    v[r] = (col && (kx != 0 || iy != 0)) ? mk(iw.x * kk / k2, iw.y * kk / k2) : mk<T>(0, 0);
                    if (owner && kx == 0 && iy == 0) v[r] = mk(f == 1 ? m0 : m1, (T)0);
                }
            }
            FFTi::run(v, j, c, buf, a.twy, 1, sync);
            cpx<T> *dst = f == 0 ? a.fa : f == 1 ? a.fx : a.fy;
            if (active) {
#pragma unroll
                for (int r = 0; r < R; r++) dst[cbase + (size_t)(j + r * TPC) * W] = v[r];
            }
        }
    }
};

}  // namespace af
