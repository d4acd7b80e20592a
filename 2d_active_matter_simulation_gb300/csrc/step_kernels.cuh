// The two fused passes of one integrating-factor RK4 stage.
//
// Reference: ActFlow_V3-2.cu (DominikSuchla/2D_active_matter_simulation).  The
// reference spends a stage on 7 cuFFT 2-D transforms and 5 pointwise kernels
// (nonl_func ActFlow_V3-2.cu:1036-1088, integrate_func_* 940-1018,
// reality_func 1228-1243).  Here a stage is two kernels:
//
//   row pass  (one CTA row group per y):   C2R along x of a, ux, uy (the
//             mean velocity added as their k = 0 mode) -> real-space products
//             P = lam' w ux + beta' |u|^2 uy, Q = lam' w uy - beta' |u|^2 ux
//             and the per-row sums of |u|^2 (energy) and |u|^2 u (mean-flow
//             right-hand side) -> R2C along x of P and Q.
//   column pass (one CTA per group of kx columns, plus one reducer CTA):
//             forward FFT along y of P, Q -> N = i (-kx P^ - ky Q^) * mask ->
//             Hermitian repair of the kx = 0 column of the accumulator -> RK
//             stage combination with the integrating factors -> Biot-Savart ->
//             inverse FFT along y of the next stage input a, ux, uy; the
//             reducer CTA sums the row sums and updates the mean-flow scalars.
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
    int outside;                           // set_state: the loaded state has a nonzero mode
                                           // outside the 1/2-rule ellipse (tile kernel)
};
static_assert(sizeof(Scalars) == 64, "the column pass copies Scalars as four 16-byte pieces");

template <typename T>
struct StepArgs {
    int nx, ny, nxh, nt;            // grid; nt = number of column tiles
    int kxp, ntp;                   // highest kx carried by the stage fields and the
                                    // number of column tiles the passes touch (pruned
                                    // transforms: kxp = Nx/4 under the 1/2 rule)
    cpx<T> *u0, *acc;               // spectral state (kx, ky): w_old / w_new
    cpx<T> *hcol;                   // w_new of the kx = 0 column, two halves of Ny
                                    // (stages alternate: one is read, the other written)
    cpx<T> *fa, *fx, *fy;           // stage input a, ux, uy in (kx, y)
    cpx<T> *P, *Q;                  // products in (kx, y)
    const cpx<T> *twx;              // exp(-2 pi i m / Nx), m < Nx
    const cpx<T> *twy;              // exp(-2 pi i m / Ny), m < Ny
    const T *kxt;                   // kx wavenumbers, nt * W entries (0 past Nx/2)
    const T *kyt;                   // ky wavenumbers in FFT order, Ny entries
    const cpx<T> *lintab;           // integrating factors {exp(L dt / 2), exp(L dt)} per (kx, ky),
                                    // tiled like the fields, computed in double and rounded
                                    // (nullptr: evaluated per value in T, as lin_func)
    T *rowp;                        // per-row sums [3][Ny]: |u|^2, |u|^2 ux, |u|^2 uy
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
    double mf_d2, mf_d6, mf_d6l, mf_d3l2;   // dt/2, dt/6, dt/6*lin_v, dt/3*lin2_v (dt as T, in double)
    double inv_2n3;                 // 1 / (2 N^3)
    int mode;                       // column pass: 0 = start from u0, 1..4 = RK stage
    int tma_field0;                 // index of this simulation's u0 among the fields of a
                                    // shared tensor map (ensemble members: 7 * member)
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

// The mask along one column ix, with the per-column part precomputed: the
// 1/2 rule keeps ky^2 <= floor((Nx^2 Ny^2 - 16 ix^2 Ny^2) / (16 Nx^2)), exactly
// the integer condition of mask_at; the reference mask keeps ix^2 + iy^2 <= rsq
// or ix^2 + (Ny - iy)^2 <= rsq.
struct ColMask {
    int mode, ny, ix2, lim;
    AF_HD ColMask(int dealias, int rsq, int nx, int ny_, int ix) : mode(dealias), ny(ny_), ix2(ix * ix), lim(rsq)
    {
        if (dealias == 1) {
            long long X = ix, NX = nx, NY = ny_;
            long long num = NX * NX * NY * NY - 16 * X * X * NY * NY;
            lim = num < 0 ? -1 : (int)(num / (16 * NX * NX));
        }
    }
    AF_HD bool keep(int iy) const
    {
        if (mode == 1) {
            int ky = iy <= ny / 2 ? iy : iy - ny;
            return ky * ky <= lim;
        }
        if (mode == 0) return ix2 + iy * iy <= lim || ix2 + (ny - iy) * (ny - iy) <= lim;
        return true;
    }
};

// Stops the compiler from moving memory accesses across this point.
AF_HD void compiler_fence() { asm volatile("" ::: "memory"); }

AF_HD float expT(float x) { return expf(x); }
AF_HD double expT(double x) { return exp(x); }
// double-float: the exponential in double, split once (only the per-value
// integrating factors use it; the default for this precision is the table)
AF_HD df expT(df x) { return df(exp((double)x)); }

#ifdef __CUDA_ARCH__
// Butterfly shuffle of a value of the state precision across a warp.
__device__ __forceinline__ float shfl_xor(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double shfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ df shfl_xor(df v, int o)
{
    return df(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
}
#endif

// One-buffer block transform: the unrolled passes, or for double-float the
// compact loop (BlockFFT::run_compact), whose code fits the instruction caches.
template <class FFT, typename T, class Buf, class Sync>
AF_HD void fft1(cpx<T> (&v)[FFT::R], int j, int c, const Buf &b, const cpx<T> *tw, int tws, Sync &&sync)
{
    if constexpr (std::is_same_v<T, df>) FFT::run_compact(v, j, c, b, tw, tws, sync);
    else FFT::run(v, j, c, b, tw, tws, sync);
}

// Tensor-map (TMA) descriptors of the row pass's three input fields -- opaque
// 128-byte CUtensorMaps encoded on the host over the tiled layout as a 4-D
// tensor {2 W floats (one 32-byte tile row), Ny rows, column tiles, fields} --
// and the split of a row's carried tiles into nbox boxes of `box` tiles (a box
// dimension holds at most 256).  A handle encodes one map per field (one
// field each); an ensemble one map over all members' fields (field index =
// member * 7 + slot[f]), with `shared` set.
struct alignas(128) TmaDesc {
    unsigned char bytes[128];
};
struct RowTma {
    TmaDesc map[3];   // fy, fx, fa: the order of the row pass's inputs
    int nbox, box;
    int shared;       // 1: map[0] covers every field, addressed by slot
    int slot[3];      // field index of fy, fx, fa within a member's fields
};
constexpr int TMA_WAIT_LIMIT = 1 << 20;   // mbarrier polls before a row gives up

#ifdef __CUDA_ARCH__
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");   // visible to the copy engine
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// One box of a 4-D tensor map into shared memory, completion counted on bar.
__device__ __forceinline__ void tma_load_4d(void *dst, const TmaDesc *map, int c0, int c1, int c2, int c3,
                                            unsigned long long *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];\n" ::"r"(smem_addr(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
        : "memory");
}
// Wait for phase `parity` of bar to complete, polling at most `limit` times.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, int limit)
{
    for (int it = 0; it < limit; it++) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
#endif

// The mean velocity, component d (the scaled mean Nx Ny <u> of the stage
// input, Scalars::m_appr, set by the column pass before).  It is the k = 0
// mode of ux and uy (nonl_subfunc_0, ActFlow_V3-2.cu:1053-1054); the row
// passes add it to Re X(kx = 0) of each row before the C2R along x, which
// adds it to every real-space value, as the unnormalised inverse transforms
// of that mode do.
template <typename T>
AF_HD T mean_velocity(const StepArgs<T> &a, int d)
{
    return (T)a.sc->m_appr[d];
}

// ------------------------------------------------------------------ row pass
// One row y per group of TPC threads; a complex FFT of length M = Nx/2 per
// real transform (the half-length real-FFT construction).  The Hermitian pairs
// X(k), X(M-k) of the C2R inputs are read straight from global memory (the
// partner read is a reversed but coalesced access), so the inputs are never
// staged in shared memory.  The forward transforms pair Z(k) with Z(M-k)
// through one shared-memory exchange.
// Launch: blockDim = ROWS * TPC, gridDim = ceil(Ny / ROWS).
template <typename T, int LOGNX>
struct RowPass {
    static constexpr int M = 1 << (LOGNX - 1);
    static constexpr int LOGM = LOGNX - 1;
    static constexpr int LOGR = 3;
    using FFTi = BlockFFT<T, LOGM, LOGR, +1>;
    using FFTf = BlockFFT<T, LOGM, LOGR, -1>;
    static constexpr int R = FFTi::R;
    static constexpr int TPC = FFTi::TPC;
    static constexpr int ROWS = TPC >= 128 ? 1 : 128 / TPC;
    static constexpr int THREADS = ROWS * TPC;
    // resident CTAs per SM requested from the compiler: caps registers at 128 (FP32) / 255 (FP64)
    static constexpr int MINB = sizeof(T) == 4 ? (THREADS >= 256 ? 2 : 4) : 1;
    static constexpr bool WARP_SYNC = false;
    // exchange slots: FP32 per-exchange XOR maps (SWZ 5), FP64 idx + idx/8
    // (conflict-free for every exchange of the 1024-point transform with
    // 16-byte accesses; idx + idx/4 gave 2x the wavefronts and 122 KB per CTA)
    using Buf = XBuf<T, 1, sizeof(T) == 4 ? 5 : 0>;
    // slot of element idx in the pairing exchange of the forward transforms:
    // unswizzled, conflict-free for its put and its reversed get
    static AF_HD int pslot(int idx) { return idx; }
    static constexpr int BUFS = (Buf::slots(M) + 7) / 8 * 8;   // complex slots per buffer

    // per row: two exchange buffers (double buffering) for each of the three
    // transforms that run in lockstep; where six do not fit in shared memory
    // -- for FP64 CTAs of 128 threads, where two CTAs per SM fit by registers,
    // where they would keep a second CTA off the SM -- each transform reuses
    // one buffer for every exchange (SINGLE: one more barrier per exchange)
    static constexpr size_t SMEM_CAP =
        (sizeof(T) == 8 && THREADS <= 128) ? (size_t)113 * 1024 : (size_t)227 * 1024;
    static constexpr int SINGLE = (size_t)ROWS * 6 * BUFS * sizeof(cpx<T>) > SMEM_CAP ? 1 : 0;
    static constexpr int NBUF = SINGLE ? 3 : 6;
    static constexpr size_t smem_bytes() { return (size_t)ROWS * NBUF * BUFS * sizeof(cpx<T>); }

    // C2R pre-processing of X(k), X(M-k): Z(k) = E + i O with
    // E = X(k) + conj X(M-k), O = (X(k) - conj X(M-k)) exp(2 pi i k / Nx)
    // (load_pairs, then pack_pairs).  A row's element kx lives at
    // row_base + (kx / W) * Ny * W + kx % W; for k = j + r TPC with TPC a
    // multiple of W that is a per-thread base plus r * TPC * Ny: one index
    // computation per transform.

    // X(k) and X(M - k) for k = j + r TPC (zero above kxp, not read).
    static AF_HD void load_pairs(cpx<T> (&A)[R], cpx<T> (&B)[R], const cpx<T> *src, int j, int y, int ny, int kxp)
    {
        constexpr int W = Tile<T>::W;
        if constexpr (TPC % W == 0) {
            const cpx<T> *pa = src + tidx<T>(j, y, ny);
            const cpx<T> *pb = src + tidx<T>(M - j, y, ny);
            const size_t stride = (size_t)(TPC / W) * ny * W;
#pragma unroll
            for (int r = 0; r < R; r++) {
                const int k = j + r * TPC;
                A[r] = k <= kxp ? pa[r * stride] : mk<T>(0, 0);
                B[r] = M - k <= kxp ? pb[-(long long)(r * stride)] : mk<T>(0, 0);
            }
        } else {
#pragma unroll
            for (int r = 0; r < R; r++) {
                const int k = j + r * TPC;
                A[r] = k <= kxp ? src[tidx<T>(k, y, ny)] : mk<T>(0, 0);
                B[r] = M - k <= kxp ? src[tidx<T>(M - k, y, ny)] : mk<T>(0, 0);
            }
        }
    }
    // The pre/post-processing twiddle W^k = exp(-2 pi i k / Nx) for
    // k = j + r TPC equals W^j * exp(-2 pi i r / (2R)) (Nx = 2 R TPC): one table
    // value per thread (wj) times a compile-time rotation.
    static AF_HD void pack_pairs(cpx<T> (&v)[R], const cpx<T> (&A)[R], const cpx<T> (&B)[R], cpx<T> wj, int j,
                                 T m)
    {
        static_for<0, R>([&](auto rc) {
            constexpr int r = decltype(rc)::value;
            cpx<T> a = A[r], b = conj(B[r]);
            if (r == 0 && j == 0) {   // X(0), X(M): imaginary parts dropped, as a half-plane C2R does
                a.y = 0;
                b.y = 0;
                a.x = a.x + m;        // the field's mean (the k = 0 mode), see mean_velocity
            }
            const cpx<T> E = a + b;
            const cpx<T> O = rot<r, 2 * R, +1>(cmulc(a - b, wj));   // (A - conj B) conj(W^k)
            v[r] = mk(E.x - O.y, E.y + O.x);
        });
    }
    // X(k) = E + W^k O for k = j + r TPC (see unpack); Bp = Z(M - k).
    template <int r>
    static AF_HD cpx<T> unpack_r(cpx<T> A, cpx<T> Bp, cpx<T> wj)
    {
        const cpx<T> B = conj(Bp);
        const cpx<T> E = scale(A + B, (T)0.5);
        const cpx<T> D = scale(A - B, (T)0.5);
        return E + rot<r, 2 * R, -1>(cmul(mk(D.y, -D.x), wj));
    }

    // Sum (t0, t1, t2) over the TPC threads of a row in T; the result is valid
    // in thread j = 0.  GPU: warp shuffles, then one shared-memory step across
    // the row's warps.  Elsewhere: a shared-memory tree.  (FP32 sums are at
    // least as accurate as the reference's own: it sums the energy sequentially
    // in float, ActFlow_V3-2.cu:1118-1124, and takes the mean-flow sums from the
    // k = 0 term of a float FFT.)
    template <class Sync>
    static AF_HD void row_sum3(T &t0, T &t1, T &t2, int j, T *scratch, Sync &&sync)
    {
#ifdef __CUDA_ARCH__
        if constexpr (TPC >= 32) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                t0 += shfl_xor(t0, o);
                t1 += shfl_xor(t1, o);
                t2 += shfl_xor(t2, o);
            }
            constexpr int NW = TPC / 32;
            sync();
            if ((j & 31) == 0) {
                scratch[(j >> 5) * 3 + 0] = t0;
                scratch[(j >> 5) * 3 + 1] = t1;
                scratch[(j >> 5) * 3 + 2] = t2;
            }
            sync();
            if (j == 0) {
                for (int w = 1; w < NW; w++) {
                    t0 += scratch[w * 3 + 0];
                    t1 += scratch[w * 3 + 1];
                    t2 += scratch[w * 3 + 2];
                }
            }
            return;
        }
#endif
        sync();
        scratch[j] = t0;
        scratch[TPC + j] = t1;
        scratch[2 * TPC + j] = t2;
        sync();
        for (int s = TPC / 2; s > 0; s >>= 1) {
            if (j < s) {
                scratch[j] += scratch[j + s];
                scratch[TPC + j] += scratch[TPC + j + s];
                scratch[2 * TPC + j] += scratch[2 * TPC + j + s];
            }
            sync();
        }
        t0 = scratch[0];
        t1 = scratch[TPC];
        t2 = scratch[2 * TPC];
    }

    // R2C post-processing: X(k) = E + exp(-2 pi i k / Nx) O with
    // E = (Z(k) + conj Z(M-k)) / 2, O = (Z(k) - conj Z(M-k)) / (2i).
    static AF_HD cpx<T> unpack(cpx<T> A, cpx<T> Bp, cpx<T> w)
    {
        cpx<T> B = conj(Bp);
        cpx<T> E = scale(A + B, (T)0.5);
        cpx<T> D = scale(A - B, (T)0.5);
        return E + cmul(mk(D.y, -D.x), w);
    }

    // Real-space products over a thread's values (uy, ux, w in v[0..2]; each
    // complex value carries two grid points): P replaces uy, Q replaces ux.
    // Then the row sums of |u|^2, |u|^2 ux, |u|^2 uy, stored by thread j = 0.
    template <class Sync>
    static AF_HD void products_and_sums(cpx<T> (&v)[3][R], const StepArgs<T> &a, int j, int y, bool active,
                                        T *scratch, Sync &&sync)
    {
        T se = 0, sx = 0, sy = 0;
        const T lam = a.lam_s, bet = a.beta_s;
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
        if constexpr (sizeof(T) == 4) {
            // the two points of a complex value as the halves of packed FP32x2
            // operations; the row sums accumulate per half and meet at the end
            float2 se2 = make_float2(0.f, 0.f), sx2 = se2, sy2 = se2;
            const float2 lam2 = make_float2(lam, lam), bet2 = make_float2(bet, bet);
#pragma unroll
            for (int r = 0; r < R; r++) {
                const float2 ux = make_float2(v[1][r].x, v[1][r].y), uy = make_float2(v[0][r].x, v[0][r].y);
                const float2 w = make_float2(v[2][r].x, v[2][r].y);
                const float2 q = __ffma2_rn(uy, uy, __fmul2_rn(ux, ux));   // |u|^2
                se2 = __fadd2_rn(se2, q);
                sx2 = __ffma2_rn(q, ux, sx2);
                sy2 = __ffma2_rn(q, uy, sy2);
                const float2 lw = __fmul2_rn(lam2, w), bq = __fmul2_rn(bet2, q);
                const float2 P2 = __ffma2_rn(bq, uy, __fmul2_rn(lw, ux));
                const float2 Q2 = __ffma2_rn(make_float2(-bq.x, -bq.y), ux, __fmul2_rn(lw, uy));
                v[0][r] = mk(P2.x, P2.y);
                v[1][r] = mk(Q2.x, Q2.y);
            }
            se = se2.x + se2.y;
            sx = sx2.x + sx2.y;
            sy = sy2.x + sy2.y;
        } else
#endif
        {
#pragma unroll
            for (int r = 0; r < R; r++) {
                T ux0 = v[1][r].x, uy0 = v[0][r].x, w0 = v[2][r].x;
                T ux1 = v[1][r].y, uy1 = v[0][r].y, w1 = v[2][r].y;
                T s0 = ux0 * ux0 + uy0 * uy0, s1 = ux1 * ux1 + uy1 * uy1;
                se += s0 + s1;
                sx += s0 * ux0 + s1 * ux1;
                sy += s0 * uy0 + s1 * uy1;
                v[0][r] = mk(lam * w0 * ux0 + bet * s0 * uy0, lam * w1 * ux1 + bet * s1 * uy1);
                v[1][r] = mk(lam * w0 * uy0 - bet * s0 * ux0, lam * w1 * uy1 - bet * s1 * ux1);
            }
        }
        row_sum3(se, sx, sy, j, scratch, sync);
        if (active && j == 0) {
            a.rowp[y] = se;
            a.rowp[a.ny + y] = sx;
            a.rowp[2 * a.ny + y] = sy;
        }
    }

    // ---- Pruned transforms at Nx = 2048: four interleaved sub-sequences.
    // With only kx <= K = Nx/4 carried (the 1/2 rule), a real row x(n) is
    // band-limited, and each sub-sequence x_s(m) = x(4m + s), s = 0..3, is the
    // real inverse transform of length K of
    //   Y_s(c) = X(c) om^{cs} + conj(X(K - c) om^{(K - c)s}),  0 < c < K,
    //   Y_s(0) = Re X(0) + 2 Re(X(K) i^s),                    om = exp(2 pi i / Nx)
    // (frequency c collects kx = c and kx = c - K).  Pairing the real outputs,
    //   z_0 = x_0 + i x_1 is the inverse transform of Z_0 = Y_0 + i Y_1,
    //   z_1 = x_2 + i x_3 that of Z_1 = Y_2 + i Y_3,
    // with Y_1 = om^c (X(c) - i conj X(K-c)), Y_2 = om^{2c} (X(c) - conj X(K-c)),
    // Y_3 = om^{3c} (X(c) + i conj X(K-c)).  So a field takes two complex
    // transforms of length K (half h = 0, 1 of the row's threads each) instead
    // of one of length M = 2K.  Forward, with Z_h the transforms of the
    // products' sub-sequence pairs (same layout), the carried outputs are
    //   X(k) = sum_s om^{-ks} Y_s(k),  0 <= k < K,   X(K) = sum_s (-i)^s Y_s(0),
    // with Y_{2h} = (Z_h(k) + conj Z_h(K-k)) / 2, Y_{2h+1} = (Z_h(k) - conj Z_h(K-k)) / 2i.
    // At Nx = 2048 the 512-point transforms take two exchanges instead of the
    // 1024-point transform's three.  Thread j = h TPQ + q holds c = q + r TPQ.
    static constexpr int K = M / 2;
    using FFTqi = BlockFFT<T, LOGM - 1, LOGR, +1>;
    using FFTqf = BlockFFT<T, LOGM - 1, LOGR, -1>;
    static constexpr int TPQ = FFTqi::TPC;
    static constexpr int QS = Buf::slots(K);   // exchange slots of one half's transform
    static constexpr bool QUARTER = !std::is_same_v<T, df> && !SINGLE && LOGNX == 11;   // FP32 and FP64

    template <class Sync>
    static AF_HD void quarter(const StepArgs<T> &a, int j, int y, bool active, const Buf (&b0)[3],
                              const Buf (&b1)[3], bool staged, Sync &&sync, T mx, T my)
    {
        static_assert(FFTqi::R == R && 2 * TPQ == TPC && FFTqf::NEXCH == 2 && TPQ % Tile<T>::W == 0 &&
                          2 * QS <= BUFS && M <= BUFS,
                      "two length-K transforms per row, radix R, two exchanges, both halves in one buffer");
        constexpr int W = Tile<T>::W;
        const int h = j / TPQ, q = j % TPQ;
        const int ny = a.ny;
        // ---- C2R of uy, ux, w: Z_h from x = X(c), xb = conj X(K - c),
        // c = q + r TPQ, in one form for both halves (s = 1 - 2h):
        //   Z_h = om^{2hc} (x + s xb) + i om^{(2h+1)c} (x - s i xb)
        // (h = 0: Z_0 = Y_0 + i Y_1; h = 1: Z_1 = Y_2 + i Y_3).  One twiddle
        // per value from the table (which holds om^{-m}), its powers by
        // products, shared by the three fields.
        cpx<T> v[3][R];
        const cpx<T> *src[3] = {a.fy, a.fx, a.fa};
        const size_t stride = (size_t)(TPQ / W) * ny * W;
        const size_t ia = tidx<T>(q, y, ny), ib = tidx<T>(K - q, y, ny);
        const T sg = h == 0 ? T(1) : T(-1);
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int c = q + r * TPQ;
            const cpx<T> t1 = ldtw(a.twx, c);                    // om^{-c}
            const cpx<T> ta = h ? cmul(t1, t1) : mk<T>(1, 0);     // om^{-2hc}
            const cpx<T> tb = h ? cmul(ta, t1) : t1;             // om^{-(2h+1)c}
#pragma unroll
            for (int f = 0; f < 3; f++) {
                cpx<T> x, bq;
                if (staged) {   // the row, kx contiguous, fetched by tensor-map copies
                    x = c <= a.kxp ? b1[f].d[c] : mk<T>(0, 0);
                    bq = K - c <= a.kxp ? b1[f].d[K - c] : mk<T>(0, 0);
                } else {
                    x = c <= a.kxp ? src[f][ia + r * stride] : mk<T>(0, 0);
                    bq = K - c <= a.kxp ? src[f][ib - r * stride] : mk<T>(0, 0);
                }
                if (r == 0 && q == 0) {   // c = 0: Y_s(0) = Re X(0) + 2 Re(X(K) i^s), Re X(0) with the mean
                    const T x0 = x.x + (f == 0 ? my : f == 1 ? mx : T(0)), bx = bq.x + bq.x, by = bq.y + bq.y;
                    v[f][0] = mk(x0 + sg * bx, x0 - sg * by);
                } else {
                    const cpx<T> xb = conj(bq);
                    const cpx<T> E = cmulc(cfma(mk(sg, sg), xb, x), ta);
                    const cpx<T> O = cmulc(cfma(mk(sg, -sg), mk(xb.y, xb.x), x), tb);
                    v[f][r] = mk(E.x - O.y, E.y + O.x);
                }
            }
        }
        const Buf qb0[3] = {Buf{b0[0].d + h * QS}, Buf{b0[1].d + h * QS}, Buf{b0[2].d + h * QS}};
        const Buf qb1[3] = {Buf{b1[0].d + h * QS}, Buf{b1[1].d + h * QS}, Buf{b1[2].d + h * QS}};
        FFTqi::template run_multi<3, 0>(v, q, 0, qb0, qb1, a.twx, 4, sync);

        // ---- products and row sums: z_h(m) = x(4m + 2h) + i x(4m + 2h + 1)
        products_and_sums(v, a, j, y, active, reinterpret_cast<T *>(b0[2].d), sync);

        // ---- R2C of P and Q; the pairing goes through b0, which the last
        // pass (reading b1) left free
        cpx<T>(&pq)[2][R] = *reinterpret_cast<cpx<T>(*)[2][R]>(&v[0]);
        const Buf pb0[2] = {qb0[0], qb0[1]};
        const Buf pb1[2] = {qb1[0], qb1[1]};
        FFTqf::template run_multi<2, 0>(pq, q, 0, pb0, pb1, a.twx, 4, sync);
#pragma unroll
        for (int f = 0; f < 2; f++)
#pragma unroll
            for (int r = 0; r < R; r++) b0[f].d[h * K + q + r * TPQ] = pq[f][r];   // Z_h(c)
        sync();
        const int kend = a.ntp * W;   // the column pass reads kx < kend
        // half h writes k = q + r TPQ for r in [h R/2, (h + 1) R/2), its own
        // Z_h(k) from registers: with S_h = Z_h(k) + conj Z_h(K-k) and
        // D_h = Z_h(k) - conj Z_h(K-k),
        //   X(k) = (S_0 + om^{-k} D_0 / i + om^{-2k} S_1 + om^{-3k} D_1 / i) / 2,
        //   X(K) = (S_0 - D_0 - S_1 + D_1) / 2  at k = 0
#pragma unroll
        for (int s = 0; s < R / 2; s++) {
            const int k = q + (s + h * (R / 2)) * TPQ;
            const int kr = (K - k) & (K - 1);
            const cpx<T> t1 = ldtw(a.twx, k), t2 = cmul(t1, t1), t3 = cmul(t2, t1);   // om^{-k}, om^{-2k}, om^{-3k}
#pragma unroll
            for (int f = 0; f < 2; f++) {
                const cpx<T> *z = b0[f].d;
                const cpx<T> own = h ? pq[f][s + R / 2] : pq[f][s];
                const cpx<T> oth = z[(1 - h) * K + k];
                const cpx<T> z0 = h ? oth : own, z1 = h ? own : oth;
                const cpx<T> z0r = conj(z[kr]), z1r = conj(z[K + kr]);
                const cpx<T> S0 = z0 + z0r, D0 = z0 - z0r, S1 = z1 + z1r, D1 = z1 - z1r;
                const cpx<T> X2 = S0 + cmul(mk(D0.y, -D0.x), t1) + cmul(S1, t2) + cmul(mk(D1.y, -D1.x), t3);
                cpx<T> *dst = f == 0 ? a.P : a.Q;
                if (active && k < kend) dst[tidx<T>(k, y, ny)] = scale(X2, (T)0.5);
                if (s == 0 && active && j == 0 && K < kend)
                    dst[tidx<T>(K, y, ny)] = scale(S0 - D0 - S1 + D1, (T)0.5);
            }
        }
#pragma unroll
        for (int f = 0; f < 2; f++) {
            cpx<T> *dst = f == 0 ? a.P : a.Q;
            for (int kx = K + 1 + j; active && kx < kend; kx += TPC) dst[tidx<T>(kx, y, ny)] = mk<T>(0, 0);
        }
    }

    // With tma (FP32): each row's three input rows are fetched by tensor-map
    // copies into that row's second set of exchange buffers (first written by
    // the transforms' second exchange), issued by the row's thread j = 0 and
    // completed on the row's mbarrier (ROWS of them at byte TMA_BAR, just past
    // the buffers); the threads then read X(k), X(M-k) from shared memory
    // instead of gathering one 8-byte value per 32-byte tile sector from
    // global memory.  A wait that runs out sets Scalars::status (the host
    // reports AM_ERR_TIMEOUT).  slot0: the simulation's first field index in
    // a shared map (StepArgs::tma_field0).
    static constexpr size_t TMA_BAR = (size_t)ROWS * NBUF * BUFS * sizeof(cpx<T>);
    static constexpr size_t smem_bytes_tma() { return TMA_BAR + ((size_t)8 * ROWS + 15) / 16 * 16; }

    template <class Sync>
    static AF_HD void body(const StepArgs<T> &a, int tid, int bid, unsigned char *smem, Sync &&sync,
                           const RowTma *tma = nullptr, int slot0 = 0)
    {
        const int rl = tid / TPC, j = tid % TPC;
        const int yy = bid * ROWS + rl;
        const bool active = yy < a.ny;
        const int y = active ? yy : a.ny - 1;   // inactive rows recompute the last row, never store
        const int ny = a.ny;
        cpx<T> *rbase = reinterpret_cast<cpx<T> *>(smem) + (size_t)rl * NBUF * BUFS;
        const Buf b0[3] = {Buf{rbase}, Buf{rbase + BUFS}, Buf{rbase + 2 * BUFS}};
        const Buf b1[3] = {Buf{rbase + (3 - 3 * SINGLE) * BUFS}, Buf{rbase + (4 - 3 * SINGLE) * BUFS},
                           Buf{rbase + (5 - 3 * SINGLE) * BUFS}};
        // the mean velocity, added to Re X(0) of ux and uy before the C2R
        const T mx = mean_velocity(a, 0), my = mean_velocity(a, 1);

        const cpx<T> *src[3] = {a.fy, a.fx, a.fa};
        if (tma) {
#ifdef __CUDA_ARCH__
            if constexpr (sizeof(T) == 4 && !SINGLE) {
                unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem + TMA_BAR) + rl;
                if (j == 0) mbar_init(bar, 1);
                sync();
                if (j == 0) {
                    mbar_expect_tx(bar, 3u * (unsigned)tma->nbox * (unsigned)tma->box * 32u);
                    for (int f = 0; f < 3; f++) {
                        const TmaDesc *m = tma->shared ? &tma->map[0] : &tma->map[f];
                        const int w = tma->shared ? slot0 + tma->slot[f] : 0;
                        for (int c = 0; c < tma->nbox; c++)
                            tma_load_4d(b1[f].d + (size_t)c * tma->box * Tile<T>::W, m, 0, y, c * tma->box, w, bar);
                    }
                }
                if (!mbar_wait(bar, 0, TMA_WAIT_LIMIT)) {
                    a.sc->status = 1;
                    mbar_wait(bar, 0, TMA_WAIT_LIMIT);   // the copies still in flight
                }
            }
#endif
        }
        if constexpr (QUARTER) {
            if (a.kxp <= K) {
                quarter(a, j, y, active, b0, b1, tma != nullptr, sync, mx, my);
                return;
            }
        }

        // ---- C2R along x of uy, ux and w, the three transforms in lockstep
        const cpx<T> wj = ldtw(a.twx, j);
        cpx<T> v[3][R];
        if (tma) {
#pragma unroll
            for (int f = 0; f < 3; f++) {
                const cpx<T> *st = b1[f].d;   // the row, kx contiguous (tile by tile)
                cpx<T> A[R], B[R];
#pragma unroll
                for (int r = 0; r < R; r++) {
                    const int k = j + r * TPC;
                    A[r] = k <= a.kxp ? st[k] : mk<T>(0, 0);
                    B[r] = M - k <= a.kxp ? st[M - k] : mk<T>(0, 0);
                }
                pack_pairs(v[f], A, B, wj, j, f == 0 ? my : f == 1 ? mx : T(0));
            }
        } else {
#pragma unroll
            for (int f = 0; f < 3; f++) {
                cpx<T> A[R], B[R];
                load_pairs(A, B, src[f], j, y, ny, a.kxp);
                pack_pairs(v[f], A, B, wj, j, f == 0 ? my : f == 1 ? mx : T(0));
            }
        }
        FFTi::template run_multi<3, SINGLE>(v, j, 0, b0, b1, a.twx, 2, sync);

        // ---- real-space products (v[f][r] holds x = 2n in its real part and
        // 2n + 1 in its imaginary part, n = j + r * TPC) and the row sums
        products_and_sums(v, a, j, y, active, reinterpret_cast<T *>(b0[2].d), sync);

        // ---- R2C along x of P and Q in lockstep; the pairing exchange of each
        // uses the buffer its transform's last pass did not read
        cpx<T>(&pq)[2][R] = *reinterpret_cast<cpx<T>(*)[2][R]>(&v[0]);
        const Buf pb0[2] = {b0[0], b0[1]};
        const Buf pb1[2] = {b1[0], b1[1]};
        FFTf::template run_multi<2, SINGLE>(pq, j, 0, pb0, pb1, a.twx, 2, sync);
        if constexpr (FFTf::NEXCH == 0 || SINGLE) sync();   // the pairing buffer may still be read
#pragma unroll
        for (int f = 0; f < 2; f++) {
            const Buf &pb = (FFTf::NEXCH & 1) ? pb1[f] : pb0[f];
#pragma unroll
            for (int r = 0; r < R; r++) pb.d[pslot(j + r * TPC)] = pq[f][r];
        }
        sync();
        const int kend = a.ntp * Tile<T>::W;   // the column pass reads kx < kend
#pragma unroll
        for (int f = 0; f < 2; f++) {
            const Buf &pb = (FFTf::NEXCH & 1) ? pb1[f] : pb0[f];
            cpx<T> *dst = f == 0 ? a.P : a.Q;
            static_for<0, R>([&](auto rc) {
                constexpr int r = decltype(rc)::value;
                const int k = j + r * TPC;
                if (active && k < kend) dst[tidx<T>(k, y, ny)] = unpack_r<r>(pq[f][r], pb.d[pslot((M - k) & (M - 1))], wj);
            });
            if (active && j == 0 && M < kend) {   // kx = M: E(0) - O(0)
                dst[tidx<T>(M, y, ny)] = unpack(pq[f][0], pq[f][0], mk<T>(-1, 0));
            }
            for (int kx = M + 1 + j; active && kx < kend; kx += TPC) dst[tidx<T>(kx, y, ny)] = mk<T>(0, 0);
        }
    }
};

template <typename T, int LOGNX>
using RowKernel = RowPass<T, LOGNX>;

// ------------------------------------- row pass, transforms in sequence
// The same work as RowPass with the transforms one after another instead of
// in lockstep: uy and ux, once transformed, wait in two shared-memory stash
// buffers while w is transformed (Q waits there while P is transformed), so
// each thread holds one transform's values at a time.  Shared memory per row:
// one exchange buffer and the two stashes; the forward transforms' pairing of
// Z(k) with Z(M-k) reads the stash that is free by then.  Launch as RowPass.
//  * FP32: radix-16 passes, TPC = M/16 threads per row (64 at Nx = 2048), two
//    exchanges per 1024-point transform instead of three, registers within
//    128; exchange slots idx + idx/16 (the map of the one-column radix-16
//    column pass).  The transform loops are unrolled.
//  * double-float: radix-8 passes, TPC = M/8 (128 at Nx = 2048), slots
//    idx + idx/8, and the transform loops NOT unrolled, so one inverse and one
//    forward transform are in the code instead of five: the lockstep kernel,
//    fully unrolled, outgrows the instruction caches (ncu at 2048^2: 5.4
//    no-instruction stall cycles per issue, 27% issue) and with 255 registers
//    and 110 KB of exchange buffers per CTA keeps 8 warps per SM.
// Nx = 512 .. 4096 (built from 1024).
template <typename T, int LOGNX>
struct RowPassS {
    static constexpr int M = 1 << (LOGNX - 1);
    static constexpr int LOGM = LOGNX - 1;
    static constexpr bool F32 = sizeof(T) == 4;
    static constexpr int LOGR = F32 ? 4 : 3;
    using FFTi = BlockFFT<T, LOGM, LOGR, +1>;
    using FFTf = BlockFFT<T, LOGM, LOGR, -1>;
    static constexpr int R = FFTi::R;
    static constexpr int TPC = FFTi::TPC;
    static_assert(TPC >= 16 && TPC % Tile<T>::W == 0, "RowPassS: Nx >= 512");
    static constexpr int ROWS = TPC >= 128 ? 1 : 128 / TPC;
    static constexpr int THREADS = ROWS * TPC;
    static constexpr int MINB = F32 || THREADS < 256 ? 4 : 2;   // 128 registers per thread at most
    using Buf = XBuf<T, 1, F32 ? 3 : 0>;
    static constexpr int BUFS = (Buf::slots(M) + 7) / 8 * 8;
    static constexpr int SLOTS = BUFS + 2 * M;    // exchange + two stashes (complex values)
    static constexpr int NW = TPC / 32 > 0 ? TPC / 32 : 1;   // warps per row
    static constexpr size_t smem_bytes()
    {
        return (size_t)ROWS * SLOTS * sizeof(cpx<T>) + (size_t)ROWS * 3 * 32 * sizeof(T);
    }
    using RP = RowPass<T, LOGNX>;

    // X(k), X(M-k) for k = j + r TPC packed into Z(k) (as RowPass::pack_pairs;
    // the twiddle of k is wj times a compile-time rotation by r / (2R) turns).
    static AF_HD void load_pack(cpx<T> (&v)[R], const cpx<T> *src, int j, int y, int ny, int kxp, cpx<T> wj, T m)
    {
        constexpr int W = Tile<T>::W;
        const cpx<T> *pa = src + tidx<T>(j, y, ny);
        const cpx<T> *pb = src + tidx<T>(M - j, y, ny);
        const size_t stride = (size_t)(TPC / W) * ny * W;
        static_for<0, R>([&](auto rc) {
            constexpr int r = decltype(rc)::value;
            const int k = j + r * TPC;
            cpx<T> a = k <= kxp ? pa[r * stride] : mk<T>(0, 0);
            cpx<T> b = M - k <= kxp ? pb[-(long long)(r * stride)] : mk<T>(0, 0);
            b = conj(b);
            if (r == 0 && j == 0) {   // X(0), X(M): imaginary parts dropped, as a half-plane C2R does
                a.y = 0;
                b.y = 0;
                a.x = a.x + m;        // the field's mean (the k = 0 mode), see mean_velocity
            }
            const cpx<T> Ev = a + b;
            const cpx<T> O = rot<r, 2 * R, +1>(cmulc(a - b, wj));
            v[r] = mk(Ev.x - O.y, Ev.y + O.x);
        });
    }

    // R2C post-processing of the row's forward transform (v, cyclic) through
    // the pairing buffer pb, stores of X(k) for k < kend.
    template <class Sync>
    static AF_HD void unpack_store(const cpx<T> (&v)[R], cpx<T> *pb, cpx<T> *dst, int j, int y, int ny, int kend,
                                   bool active, cpx<T> wj, Sync &&sync)
    {
#pragma unroll
        for (int r = 0; r < R; r++) pb[j + r * TPC] = v[r];
        sync();
        static_for<0, R>([&](auto rc) {
            constexpr int r = decltype(rc)::value;
            const int k = j + r * TPC;
            if (active && k < kend) {
                // X(k) = E + W^k O with W^k = wj exp(-2 pi i r / (2R))
                const cpx<T> B = conj(pb[(M - k) & (M - 1)]);
                const cpx<T> E = scale(v[r] + B, (T)0.5);
                const cpx<T> D = scale(v[r] - B, (T)0.5);
                dst[tidx<T>(k, y, ny)] = E + rot<r, 2 * R, -1>(cmul(mk(D.y, -D.x), wj));
            }
        });
        if (active && j == 0 && M < kend) dst[tidx<T>(M, y, ny)] = RP::unpack(v[0], v[0], mk<T>(-1, 0));
        for (int kx = M + 1 + j; active && kx < kend; kx += TPC) dst[tidx<T>(kx, y, ny)] = mk<T>(0, 0);
    }

    template <class Sync>
    static AF_HD void body(const StepArgs<T> &a, int tid, int bid, unsigned char *smem, Sync &&sync)
    {
        static_assert(R == (F32 ? 16 : 8), "radix 16 (FP32) / 8 (double-float)");
        const int rl = tid / TPC, j = tid % TPC;
        const int yy = bid * ROWS + rl;
        const bool active = yy < a.ny;
        const int y = active ? yy : a.ny - 1;   // inactive rows recompute the last row, never store
        const int ny = a.ny;
        cpx<T> *base = reinterpret_cast<cpx<T> *>(smem) + (size_t)rl * SLOTS;
        const Buf xb{base};
        cpx<T> *s1 = base + BUFS;   // uy, then Q, then Q^ for its pairing
        cpx<T> *s2 = s1 + M;        // ux, then P^ for its pairing
        T *scr = reinterpret_cast<T *>(reinterpret_cast<cpx<T> *>(smem) + (size_t)ROWS * SLOTS) + rl * 3 * 32;
        const cpx<T> wj = ldtw(a.twx, j);
        const T mx = mean_velocity(a, 0), my = mean_velocity(a, 1);   // added to Re X(0) of ux, uy

        // ---- C2R along x of uy and ux (stashed), then w (kept in registers)
        cpx<T> v[R];
#pragma unroll(F32 ? 3 : 1)
        for (int f = 0; f < 3; f++) {
            load_pack(v, f == 0 ? a.fy : f == 1 ? a.fx : a.fa, j, y, ny, a.kxp, wj, f == 0 ? my : f == 1 ? mx : T(0));
            fft1<FFTi>(v, j, 0, xb, a.twx, 2, sync);
            if (f < 2) {
                cpx<T> *st = f == 0 ? s1 : s2;
#pragma unroll
                for (int r = 0; r < R; r++) st[j + r * TPC] = v[r];
            }
        }

        // ---- real-space products (each thread reads and writes only its own
        // stash slots): P to v, Q to s1
        T se = 0, sx = 0, sy = 0;
        const T lam = a.lam_s, bet = a.beta_s;
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
        if constexpr (std::is_same_v<T, df>) {
            // double-float: the two points of a complex value as the two lanes
            // of packed double-float operations (as the FP32 lockstep pass);
            // the row sums accumulate per lane and meet at the end
            const df2 zero = df2_of(df(0), df(0));
            df2 se2 = zero, sx2 = zero, sy2 = zero;
            const df2 lam2 = df2_of(lam, lam), bet2 = df2_of(bet, bet);
#pragma unroll
            for (int r = 0; r < R; r++) {
                const cpx<T> uyv = s1[j + r * TPC], uxv = s2[j + r * TPC], wv = v[r];
                const df2 ux = df2_of(uxv.x, uxv.y), uy = df2_of(uyv.x, uyv.y), w = df2_of(wv.x, wv.y);
                const df2 q = df2_add(df2_mul(ux, ux), df2_mul(uy, uy));   // |u|^2
                se2 = df2_add(se2, q);
                sx2 = df2_add(sx2, df2_mul(q, ux));
                sy2 = df2_add(sy2, df2_mul(q, uy));
                const df2 lw = df2_mul(lam2, w), bq = df2_mul(bet2, q);
                v[r] = df2_cpx(df2_add(df2_mul(lw, ux), df2_mul(bq, uy)));
                s1[j + r * TPC] = df2_cpx(df2_add(df2_mul(lw, uy), df2_neg(df2_mul(bq, ux))));
            }
            se = df2_first(se2) + df2_second(se2);
            sx = df2_first(sx2) + df2_second(sx2);
            sy = df2_first(sy2) + df2_second(sy2);
        } else
#endif
        {
#pragma unroll
            for (int r = 0; r < R; r++) {
                const cpx<T> uyv = s1[j + r * TPC], uxv = s2[j + r * TPC], wv = v[r];
                const T ux0 = uxv.x, uy0 = uyv.x, w0 = wv.x, ux1 = uxv.y, uy1 = uyv.y, w1 = wv.y;
                const T q0 = ux0 * ux0 + uy0 * uy0, q1 = ux1 * ux1 + uy1 * uy1;
                se += q0 + q1;
                sx += q0 * ux0 + q1 * ux1;
                sy += q0 * uy0 + q1 * uy1;
                v[r] = mk(lam * w0 * ux0 + bet * q0 * uy0, lam * w1 * ux1 + bet * q1 * uy1);
                s1[j + r * TPC] = mk(lam * w0 * uy0 - bet * q0 * ux0, lam * w1 * uy1 - bet * q1 * ux1);
            }
        }
        {
            T t0 = se, t1 = sx, t2 = sy;
            row_sum3(t0, t1, t2, j, scr, sync);
            if (active && j == 0) {
                a.rowp[y] = t0;
                a.rowp[ny + y] = t1;
                a.rowp[2 * ny + y] = t2;
            }
        }

        // ---- R2C along x of P (pairing through s2, free since the products)
        // and of Q (pairing through s1, which each thread has read back)
        const int kend = a.ntp * Tile<T>::W;   // the column pass reads kx < kend
#pragma unroll(F32 ? 2 : 1)
        for (int f = 0; f < 2; f++) {
            if (f == 1) {
#pragma unroll
                for (int r = 0; r < R; r++) v[r] = s1[j + r * TPC];
            }
            // (Q: the transform's entry barrier orders the reads of s1 before
            // unpack_store's writes to it)
            fft1<FFTf>(v, j, 0, xb, a.twx, 2, sync);
            unpack_store(v, f == 0 ? s2 : s1, f == 0 ? a.P : a.Q, j, y, ny, kend, active, wj, sync);
        }
    }

    // Sum (t0, t1, t2) over the TPC threads of a row; valid in thread j = 0.
    template <class Sync>
    static AF_HD void row_sum3(T &t0, T &t1, T &t2, int j, T *scratch, Sync &&sync)
    {
#ifdef __CUDA_ARCH__
        if constexpr (TPC >= 32) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                t0 += shfl_xor(t0, o);
                t1 += shfl_xor(t1, o);
                t2 += shfl_xor(t2, o);
            }
            if ((j & 31) == 0) {
                scratch[(j >> 5) * 3 + 0] = t0;
                scratch[(j >> 5) * 3 + 1] = t1;
                scratch[(j >> 5) * 3 + 2] = t2;
            }
            sync();
            if (j == 0) {
                for (int w = 1; w < NW; w++) {
                    t0 += scratch[w * 3 + 0];
                    t1 += scratch[w * 3 + 1];
                    t2 += scratch[w * 3 + 2];
                }
            }
            return;
        }
#endif
        // elsewhere (and for rows of fewer than 32 threads): thread 0 adds the
        // row's values in thread order
        for (int q = 0; q < TPC; q++) {
            if (j == q) {
                if (q == 0) {
                    scratch[0] = t0;
                    scratch[1] = t1;
                    scratch[2] = t2;
                } else {
                    scratch[0] += t0;
                    scratch[1] += t1;
                    scratch[2] += t2;
                }
            }
            sync();
        }
        t0 = scratch[0];
        t1 = scratch[1];
        t2 = scratch[2];
    }
};

// ------------------------------------------------- sums over the row sums
// Compensated ("float-float") accumulation for the FP32 path: hi + lo carries
// about 44 significant bits, so the sum over all rows is as good as a double
// sum while it stays on the FP32 pipes (FP64 throughput on this GPU is a small
// fraction of FP32).  Two-sum after Knuth, TAOCP vol. 2, 4.2.2, theorem B.
// The order of summation is fixed, so results are reproducible bit for bit.
template <typename T>
struct RowAcc {   // FP64 path: plain double
    double v = 0;
    AF_HD void add(T x) { v += (double)x; }
    AF_HD void add(const RowAcc &o) { v += o.v; }
    AF_HD double value() const { return v; }
#ifdef __CUDA_ARCH__
    __device__ void add_xor(int o) { v += __shfl_xor_sync(0xffffffffu, v, o); }
#endif
};
template <>
struct RowAcc<float> {
    float hi = 0, lo = 0;
    AF_HD void add2(float bh, float bl)
    {
        const float s = hi + bh;
        const float bb = s - hi;
        float e = (hi - (s - bb)) + (bh - bb);
        e += lo + bl;
        hi = s + e;
        lo = e - (hi - s);
    }
    AF_HD void add(float x) { add2(x, 0.f); }
    AF_HD void add(const RowAcc &o) { add2(o.hi, o.lo); }
    AF_HD double value() const { return (double)hi + (double)lo; }
#ifdef __CUDA_ARCH__
    __device__ void add_xor(int o)
    {
        const float h = __shfl_xor_sync(0xffffffffu, hi, o), l = __shfl_xor_sync(0xffffffffu, lo, o);
        add2(h, l);
    }
#endif
};
template <>
struct RowAcc<df> {   // double-float path: the sums in double-float
    df v{};
    AF_HD void add(df x) { v += x; }
    AF_HD void add(const RowAcc &o) { v += o.v; }
    AF_HD double value() const { return (double)v; }
#ifdef __CUDA_ARCH__
    __device__ void add_xor(int o) { v += shfl_xor(v, o); }
#endif
};

// 16-byte global -> shared copy that completes asynchronously (the thread
// that issued it waits with cp_async_wait_all before reading the data).
AF_HD void cp_async16(void *dst_smem, const void *src)
{
#ifdef __CUDA_ARCH__
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
#else
    for (int i = 0; i < 16; i++) static_cast<unsigned char *>(dst_smem)[i] = static_cast<const unsigned char *>(src)[i];
#endif
}
AF_HD void cp_async8(void *dst_smem, const void *src)
{
#ifdef __CUDA_ARCH__
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
#else
    for (int i = 0; i < 8; i++) static_cast<unsigned char *>(dst_smem)[i] = static_cast<const unsigned char *>(src)[i];
#endif
}
// A load cached in L2 only: for values read once, so that they do not evict
// the lines prefetched into L1 for later use.
template <typename T>
AF_HD cpx<T> ld_stream(const cpx<T> *p)
{
#ifdef __CUDA_ARCH__
    cpx<T> r;
    if constexpr (sizeof(cpx<T>) == 8) {
        const float2 v = __ldcg(reinterpret_cast<const float2 *>(p));
        memcpy(&r, &v, sizeof r);
    } else {
        const float4 v = __ldcg(reinterpret_cast<const float4 *>(p));
        memcpy(&r, &v, sizeof r);
    }
    return r;
#else
    return *p;
#endif
}
// Hint to bring the line holding p into this SM's L1 (no register, no wait).
AF_HD void prefetch_l1(const void *p)
{
#ifdef __CUDA_ARCH__
    asm volatile("prefetch.global.L1 [%0];\n" ::"l"(p));
#else
    (void)p;
#endif
}
// Named barrier 1 (barrier 0 is __syncthreads): bar_arrive signals without
// waiting, bar_wait waits until `n` threads have arrived or waited; prior
// shared-memory writes of the arriving threads are visible after the wait.
AF_HD void bar_arrive1(int n)
{
#ifdef __CUDA_ARCH__
    asm volatile("bar.arrive 1, %0;\n" ::"r"(n) : "memory");
#else
    (void)n;
#endif
}
AF_HD void bar_wait1(int n)
{
#ifdef __CUDA_ARCH__
    asm volatile("bar.sync 1, %0;\n" ::"r"(n) : "memory");
#else
    (void)n;
#endif
}
AF_HD void cp_async_commit()
{
#ifdef __CUDA_ARCH__
    asm volatile("cp.async.commit_group;\n" ::: "memory");
#endif
}
AF_HD void cp_async_wait_all()
{
#ifdef __CUDA_ARCH__
    asm volatile("cp.async.wait_all;\n" ::: "memory");
#endif
}

// --------------------------------------------------------------- column pass
// CW adjacent kx columns per group of CW * TPC threads (lane c = column in the
// group, j = thread of that column's transform), TILES groups per CTA.  Three
// launch shapes (VAR), chosen per precision and Ny at run time (see
// col_variant, am_autotune):
//  * wide (VAR 0): CW = W, a whole tile per group, so every store covers
//    whole 32-byte sectors (FP32 at Ny = 4096 takes half a tile, 512 threads,
//    to stay within 128 registers).  Radix 16 (FP32) / 8 (FP64).
//  * narrow (VAR 1): CW = 1, one column per group: CTAs of 128 threads
//    (FP32, Ny <= 2048), up to four per SM, each synchronising only its own
//    warps.  Stores then cover a quarter sector each, which at 2048 cost more
//    (ncu: 4x the L2 write sectors, 36 -> 47 us) than the extra CTAs won;
//    below it the smaller CTAs win (ragged batch of 128^2..1024^2 grids
//    +14%).
//  * wide radix 8 (VAR 2, FP32 only): radix-8 passes with twice the threads
//    per column (8 values each, 64 registers): one more exchange per
//    transform, twice the warps per SM to hide the latency of a pass that is
//    latency-bound with one 512-thread CTA per SM.  CTAs of at most 512
//    threads, so at Ny = 2048 a CTA takes half a tile (two columns) and two
//    independent CTAs share an SM, their load and transform phases
//    interleaving (31.1 -> 29.3 us, though its stores cover half sectors);
//    at 4096 a CTA takes half a tile with 1024 threads (512 would leave one
//    column per CTA: 132 -> 153 us).
// MODE 0 starts from u0 (after set_state), MODE 1..4 is the RK stage.
// Launch: blockDim = THREADS, gridDim = ceil(columns carried / COLS).
template <typename T, int LOGNY, int MODE, int VAR = (LOGNY < 11 ? 1 : 0)>
struct ColPass {
    static constexpr bool NARROW = VAR == 1;
    // threads per CTA at most: 512, except the radix-8 shape at Ny = 4096
    // (1024: a half tile per CTA; with 512 threads each CTA would take a
    // single column and store quarter sectors)
    static constexpr int TMAX = VAR == 2 && LOGNY >= 12 ? 1024 : 512;
    static constexpr int W = Tile<T>::W;
    static constexpr int LOGR = sizeof(T) == 4 && VAR != 2 ? 4 : 3;
    using FFTf = BlockFFT<T, LOGNY, LOGR, -1>;
    using FFTi = BlockFFT<T, LOGNY, LOGR, +1>;
    static constexpr int R = FFTf::R;
    static constexpr int TPC = FFTf::TPC;
    static constexpr int L = 1 << LOGNY;
    static constexpr int CW = NARROW ? 1 : (W * TPC <= TMAX ? W : (TMAX / TPC > 1 ? TMAX / TPC : 1));
    static constexpr int TILES = CW * TPC >= 128 ? 1 : 128 / (CW * TPC);   // column groups per CTA
    static constexpr int THREADS = TILES * CW * TPC;
    static constexpr int COLS = TILES * CW;                                // columns per CTA
    // CTAs per SM the registers allow (128 per thread at most; VAR 2: 64)
    static constexpr int MCAP = VAR == 2 ? 8 : 4;
    static constexpr int TREG = VAR == 2 ? 1024 : 512;   // threads per SM the registers are budgeted for
    static constexpr int MINB = THREADS >= TREG ? 1 : (TREG / THREADS > MCAP ? MCAP : TREG / THREADS);
    // exchange slots: CW columns interleaved, idx + idx/8; one column: idx +
    // idx/16 (FP32) / idx + idx/8 (FP64), conflict-free for every pass of
    // these transforms (simulated bank pattern)
    using Buf = XBuf<T, CW, (CW == 1 && sizeof(T) == 4) ? 3 : 0>;
    static constexpr int BUFS = (Buf::slots(L) + 7) / 8 * 8;
    // Shared memory, within MINB CTAs per SM: the exchange buffers; then what
    // CTA 0 (holding column kx = 0) fetches at kernel start in stages 1-4 so
    // that its extra work (the Hermitian repair, the step counters) runs from
    // shared memory: the Scalars, then the source of the kx = 0 column's
    // mirror values (each where it fits); then one partial sum per warp (the
    // reducer CTA's row-sum reduction).
    static constexpr size_t XB = (size_t)TILES * BUFS * sizeof(cpx<T>);
    static constexpr size_t SCB = sizeof(Scalars);
    static constexpr size_t MIB = (size_t)L * sizeof(cpx<T>);
    static constexpr int NW = THREADS / 32 > 0 ? THREADS / 32 : 1;
    static constexpr size_t WPB = (size_t)3 * NW * sizeof(RowAcc<T>);
    static constexpr size_t LIM = (size_t)228 * 1024 / MINB - 1024 < (size_t)227 * 1024
                                      ? (size_t)228 * 1024 / MINB - 1024
                                      : (size_t)227 * 1024;
    // The radix-8 shape at Ny >= 4096 stages only the Scalars: CTA 0
    // prefetches the mirror column into L1 instead, because every CTA of the
    // launch would reserve that buffer, and the shared-memory carve-out it
    // takes comes out of the L1 that holds the stage inputs prefetched during
    // Q's transform (4096^2: column pass 131 -> 122 us with the mirror and the
    // row sums out of shared memory; at 2048 neutral).
    static constexpr bool OWN = !(VAR == 2 && LOGNY >= 12);
    static constexpr bool PS = XB + SCB + WPB <= LIM;                   // Scalars
    static constexpr bool PM = OWN && PS && XB + SCB + MIB + WPB <= LIM;  // + mirror column
    static constexpr size_t O_SC = XB, O_MI = O_SC + SCB;
    static constexpr size_t O_WP = O_MI + (PM ? MIB : 0);
    static constexpr int CE = 16 / (int)sizeof(T);                     // row sums per 16-byte read

    static constexpr size_t smem_bytes() { return O_WP + WPB; }

    // CTAs of a launch: the column groups, then one more, the reducer, which
    // carries no columns (launch sites: grid = ctas(a)).
    static AF_HD int col_ctas(const StepArgs<T> &a) { return (a.ntp * W + COLS - 1) / COLS; }
    static AF_HD int ctas(const StepArgs<T> &a) { return col_ctas(a) + 1; }

    // The reducer CTA: the energy and the mean-flow right-hand side from the
    // row sums (compensated sums, about double accuracy; the reference sums
    // the energy in float on the host, ActFlow_V3-2.cu:1118-1124), and the
    // mean-flow scalar update of this stage -- -beta' Re F[|u|^2 u](0)
    // (ActFlow_V3-2.cu:1086-1087) and its stage updates (ActFlow_V3-2.cu:
    // 729-732, 756-759, 778-781, 799-802, 820-821).  Its own CTA keeps this
    // serial work off the column groups' critical path; the next row pass
    // adds the updated mean velocity m_appr in real space.  It writes only
    // m_old, m_new, m_appr and the energy (CTA 0 owns step and nan_step).
    template <class Sync>
    static AF_HD void reduce_scalars(const StepArgs<T> &a, int tid, unsigned char *smem, Sync &&sync)
    {
        RowAcc<T> *wp = reinterpret_cast<RowAcc<T> *>(smem + O_WP);   // warp partials
        const int ny = a.ny;
        RowAcc<T> sum[3];
        if constexpr (MODE != 0) {
#pragma unroll
            for (int k = 0; k < 3; k++)
                for (int q = tid; q < ny / CE; q += THREADS) {
                    const T *src = a.rowp + (size_t)k * ny + q * CE;
#pragma unroll
                    for (int e = 0; e < CE; e++) sum[k].add(src[e]);
                }
        }
        block_sum3(sum, tid, wp, sync);
        if (tid == 0) {
            Scalars *g = a.sc;
            double m_old[2] = {g->m_old[0], g->m_old[1]}, m_new[2] = {g->m_new[0], g->m_new[1]};
            double m_appr[2] = {g->m_appr[0], g->m_appr[1]};
            const double red[3] = {sum[0].value(), sum[1].value(), sum[2].value()};
            // (the dt factors come precomputed from the host: no FP64
            // division on this serial path)
            const double n0 = -a.beta_sd * red[1], n1 = -a.beta_sd * red[2];
            const double dd = (double)a.dt;
            if constexpr (MODE == 0) {
                for (int d = 0; d < 2; d++) m_old[d] = m_appr[d] = m_new[d];
            } else if constexpr (MODE == 1) {
                a.energy[g->step % a.ecap] = red[0] * a.inv_2n3;
                m_new[0] += a.mf_d6l * n0;
                m_new[1] += a.mf_d6l * n1;
                m_appr[0] = a.lin2_v * (m_old[0] + a.mf_d2 * n0);
                m_appr[1] = a.lin2_v * (m_old[1] + a.mf_d2 * n1);
            } else if constexpr (MODE == 2) {
                m_new[0] += a.mf_d3l2 * n0;
                m_new[1] += a.mf_d3l2 * n1;
                m_appr[0] = a.lin2_v * (m_old[0] + a.mf_d2 * n0);
                m_appr[1] = a.lin2_v * (m_old[1] + a.mf_d2 * n1);
            } else if constexpr (MODE == 3) {
                m_new[0] += a.mf_d3l2 * n0;
                m_new[1] += a.mf_d3l2 * n1;
                m_appr[0] = a.lin_v * (m_old[0] + dd * n0);
                m_appr[1] = a.lin_v * (m_old[1] + dd * n1);
            } else {
                m_new[0] += a.mf_d6 * n0;
                m_new[1] += a.mf_d6 * n1;
                for (int d = 0; d < 2; d++) m_old[d] = m_appr[d] = m_new[d];
            }
            for (int d = 0; d < 2; d++) {
                g->m_old[d] = m_old[d];
                g->m_new[d] = m_new[d];
                g->m_appr[d] = m_appr[d];
            }
        }
    }

    template <class Sync>
    static AF_HD void body(const StepArgs<T> &a, int tid, int bid, unsigned char *smem, Sync &&sync)
    {
        if (bid == col_ctas(a)) {   // the reducer (uniform over the CTA)
            reduce_scalars(a, tid, smem, sync);
            return;
        }
        const int tl = tid / (CW * TPC);
        const int rem = tid % (CW * TPC);
        const int c = rem % CW, j = rem / CW;
        const int kx = (bid * TILES + tl) * CW + c;   // this thread's column
        const bool active = kx < a.ntp * W;
        const int tile = kx / W;                  // its tile in the HBM layout
        const bool col = active && kx <= a.kxp;   // a column that carries data
        const int ny = a.ny, nx = a.nx;
        Buf buf{reinterpret_cast<cpx<T> *>(smem) + (size_t)tl * BUFS};
        const Scalars *ssm = reinterpret_cast<const Scalars *>(smem + O_SC);   // owner copies
        cpx<T> *mir = reinterpret_cast<cpx<T> *>(smem + O_MI);
        const bool owner = bid == 0;   // this CTA holds column kx = 0
        const T kxv = active ? a.kxt[kx] : (T)0;
        const size_t cbase = active ? (size_t)tile * ny * W + kx % W : 0;
        const T dt = a.dt;
        // The kx = 0 column keeps w_new in a.hcol: stage 1 writes half 0,
        // stage 2 reads 0 and writes 1, stage 3 reads 1 and writes 0, stage 4
        // reads 0.  So the Hermitian repair can read the mirror values
        // w_new(-ky) while this stage writes its results, without a barrier.
        const cpx<T> *hin = a.hcol + (size_t)(MODE & 1) * ny;
        cpx<T> *hout = a.hcol + (size_t)((MODE + 1) & 1) * ny;

        // The owner fetches its extra inputs now.  The Scalars (their step
        // counters) are read by thread 0 and the mirror column by the kx = 0
        // column's threads, both after the barriers of the forward transforms.
        if constexpr (MODE != 0 && PS) {
            if (owner) {
                if (tid < 4) cp_async16(smem + O_SC + 16 * tid, reinterpret_cast<const unsigned char *>(a.sc) + 16 * tid);
                if constexpr (PM && MODE == 1) {   // w_old of the kx = 0 column (tile 0, lane 0)
                    for (int y = tid; y < ny; y += THREADS) {
                        if constexpr (sizeof(cpx<T>) == 8) cp_async8(mir + y, a.u0 + (size_t)y * W);
                        else cp_async16(mir + y, a.u0 + (size_t)y * W);
                    }
                } else if constexpr (PM) {
                    constexpr int CC = 16 / (int)sizeof(cpx<T>);
                    for (int q = tid; q < ny / CC; q += THREADS) cp_async16(mir + q * CC, hin + q * CC);
                }
                cp_async_commit();
                if constexpr (!PM) {   // the mirror source: four tile rows per line (MODE 1), or hin
                    if constexpr (MODE == 1) {
                        for (int q = tid; q < ny / 4; q += THREADS) prefetch_l1(a.u0 + (size_t)(4 * q) * W);
                    } else {
                        constexpr int HL = 128 / (int)sizeof(cpx<T>);
                        for (int q = tid; q < ny / HL; q += THREADS) prefetch_l1(hin + (size_t)q * HL);
                    }
                }
            }
        }

        // ---- forward FFT along y of P and Q, N = i (-kx P^ - ky Q^) * mask
        cpx<T> nl[R];
        if constexpr (MODE != 0) {
            cpx<T> ph[R], v[R];
#pragma unroll
            for (int r = 0; r < R; r++) v[r] = active ? ld_stream(a.P + cbase + (size_t)(j + r * TPC) * W) : mk<T>(0, 0);
            fft1<FFTf>(v, j, c, buf, a.twy, 1, sync);
#pragma unroll
            for (int r = 0; r < R; r++) ph[r] = v[r];
#pragma unroll
            for (int r = 0; r < R; r++) v[r] = active ? ld_stream(a.Q + cbase + (size_t)(j + r * TPC) * W) : mk<T>(0, 0);
            // the stage's inputs move towards L1 while Q is transformed
            if (active) {
#pragma unroll
                for (int r = 0; r < R; r++) {
                    const size_t g = cbase + (size_t)(j + r * TPC) * W;
                    if constexpr (MODE != 4) prefetch_l1(a.u0 + g);
                    if constexpr (MODE >= 2) prefetch_l1(a.acc + g);
                    if constexpr (MODE != 4) {
                        if (a.lintab) prefetch_l1(a.lintab + g);
                    }
                }
            }
            if constexpr (PS) {
                // the owner's copies are complete; the barrier that starts the
                // next transform makes them visible to the whole CTA
                if (owner) {
                    cp_async_wait_all();
                    if constexpr (FFTf::NEXCH == 0) sync();
                }
            }
            fft1<FFTf>(v, j, c, buf, a.twy, 1, sync);
            const ColMask cm(a.dealias, a.rsq, nx, ny, kx);
#pragma unroll
            for (int r = 0; r < R; r++) {
                int iy = j + r * TPC;
                T kyv = a.kyt[iy];
                T m = (col && cm.keep(iy)) ? (T)1 : (T)0;
                if constexpr (std::is_same_v<T, df>) {   // complex operations, packed pipe
                    const cpx<T> t = scale(ph[r], -kxv) + scale(v[r], -kyv);   // (tr, ti)
                    nl[r] = scale(mk(-t.y, t.x), m);
                } else {
                    T tr = -kxv * ph[r].x - kyv * v[r].x;
                    T ti = -kxv * ph[r].y - kyv * v[r].y;
                    nl[r] = mk(-ti * m, tr * m);
                }
            }
        }

        // ---- RK stage combination (integrate_func_0..4, ActFlow_V3-2.cu:940-1018)
        // with the Hermitian repair of the accumulator's kx = 0 column before the
        // addition (reality_func, ActFlow_V3-2.cu:1228-1243).  Its loads are
        // issued before the owner's mean-flow work so that their latency
        // overlaps it.
        cpx<T> av[R], accv[R];
        const bool c0 = owner && tl == 0 && c == 0;   // the kx = 0 column
        if constexpr (MODE == 0) {
#pragma unroll
            for (int r = 0; r < R; r++) av[r] = active ? a.u0[cbase + (size_t)(j + r * TPC) * W] : mk<T>(0, 0);
        } else {
#pragma unroll
            for (int r = 0; r < R; r++) {
                size_t g = cbase + (size_t)(j + r * TPC) * W;
                if constexpr (MODE == 1) {
                    av[r] = active ? a.u0[g] : mk<T>(0, 0);   // w_old
                } else {
                    accv[r] = c0 ? hin[j + r * TPC] : active ? a.acc[g] : mk<T>(0, 0);
                    if constexpr (MODE != 4) av[r] = active ? a.u0[g] : mk<T>(0, 0);
                }
            }
        }

        // ---- step counters for the NaN probe (thread 0 of the owner, stage 4;
        // the reducer CTA updates the mean-flow scalars and the energy)
        int sc_step = 0, sc_nan = 0;
        if constexpr (MODE == 4) {
            if (owner && tid == 0) {
                const Scalars *sv = PS ? ssm : a.sc;
                sc_step = sv->step;
                sc_nan = sv->nan_step;
            }
        }

        if constexpr (MODE != 0) {
#pragma unroll
            for (int r = 0; r < R; r++) {
                const int iy = j + r * TPC;
                const size_t g = cbase + (size_t)iy * W;
                const cpx<T> n = nl[r], o = av[r];
                // e2 = exp(L dt / 2) and e1 = exp(L dt) at (kx, ky): from the
                // table (double, rounded once), or e2 evaluated here in T and
                // e1 formed as its square.  ky(-iy) = -ky(iy) exactly, so the
                // mirror shares these values.
                T e2 = 0, e1 = 0;
                if constexpr (MODE != 4) {
                    if (a.lintab) {
                        const cpx<T> f = active ? a.lintab[g] : mk<T>(0, 0);
                        e2 = f.x;
                        e1 = f.y;
                    } else {
                        e2 = lin_at(a, kxv, iy, dt / 2);
                        e1 = e2 * e2;
                    }
                }
                cpx<T> w = MODE == 1 ? scale(o, e1) : accv[r];   // stage 1: w_new = w_old * lin
                if (c0 && iy != 0 && iy != ny / 2) {
                    // Hermitian repair with the mirror value w_new(-ky)
                    const int my = ny - iy;
                    cpx<T> b;
                    if constexpr (MODE == 1) b = scale(PM ? mir[my] : a.u0[cbase + (size_t)my * W], e1);
                    else b = PM ? mir[my] : hin[my];
                    if (iy < ny / 2) w = mk((T)0.5f * (w.x + b.x), (T)0.5f * (w.y - b.y));
                    else w = conj(mk((T)0.5f * (b.x + w.x), (T)0.5f * (b.y - w.y)));
                }
                if constexpr (MODE == 1) {
                    T f = dt / 6 * e1;
                    w = axpy(w, f, n);
                    av[r] = scale(axpy(o, dt / 2, n), e2);
                } else if constexpr (MODE == 2) {
                    T f = dt / 3 * e2;
                    w = axpy(w, f, n);
                    av[r] = scale(axpy(o, dt / 2, n), e2);
                } else if constexpr (MODE == 3) {
                    T f = dt / 3 * e2;
                    w = axpy(w, f, n);
                    av[r] = scale(axpy(o, dt, n), e1);
                } else {
                    w = axpy(w, dt / 6, n);
                    av[r] = w;   // next step: w_old = w_appr = w_new
                }
                if (active) {
                    if constexpr (MODE == 4) a.u0[g] = w;
                    else if (c0) hout[iy] = w;
                    else a.acc[g] = w;
                }
            }
            if constexpr (MODE == 4) {
                if (owner && tid == 0) {
                    // NaN probe on Re w(0,0) (check_func, ActFlow_V3-2.cu:884-897).
                    if (av[0].x != av[0].x && sc_nan < 0) a.sc->nan_step = sc_step;
                    a.sc->step = sc_step + 1;
                }
            }
        }

        // ---- Biot-Savart (nonl_subfunc_0, ActFlow_V3-2.cu:1176-1180), then the
        // inverse FFT along y of a, ux, uy.  The k = 0 slot of ux, uy (the mean
        // velocity, ActFlow_V3-2.cu:1053-1054) stays zero here: the next row
        // pass adds the mean to every real-space value instead.
#pragma unroll 1
        for (int f = 0; f < 3; f++) {
            cpx<T> v[R];
#pragma unroll
            for (int r = 0; r < R; r++) {
                const int iy = j + r * TPC;
                const cpx<T> w = av[r];
                if (f == 0) {
                    v[r] = col ? w : mk<T>(0, 0);
                } else {
                    const T kyv = a.kyt[iy];
                    const T k2 = kyv * kyv + kxv * kxv;
                    const T q = (f == 1 ? kyv : -kxv) / k2;
                    cpx<T> u;
                    if constexpr (std::is_same_v<T, df>) u = scale(mk(-w.y, w.x), q);   // packed pipe
                    else u = mk(-w.y * q, w.x * q);
                    v[r] = (col && (kx != 0 || iy != 0)) ? u : mk<T>(0, 0);   // k = 0: the mean, added by the row pass
                }
            }
            fft1<FFTi>(v, j, c, buf, a.twy, 1, sync);
            cpx<T> *dst = f == 0 ? a.fa : f == 1 ? a.fx : a.fy;
            if (active) {
#pragma unroll
                for (int r = 0; r < R; r++) dst[cbase + (size_t)(j + r * TPC) * W] = v[r];
            }
        }
    }

    // Sum the three accumulators over the CTA; the result is valid in thread 0.
    // GPU: warp shuffles, one partial per warp in shared memory; warps 1.. go
    // on after leaving their partial (named barrier, arrive only), warp 0 waits
    // for them and combines the partials with shuffles.  Elsewhere: the
    // partials from a per-warp loop, then thread 0 adds them in warp order.
    template <class Sync>
    static AF_HD void block_sum3(RowAcc<T> (&sum)[3], int tid, RowAcc<T> *wp, Sync &&sync)
    {
#ifdef __CUDA_ARCH__
        static_assert(NW <= 32, "one partial per lane of warp 0");
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int k = 0; k < 3; k++) sum[k].add_xor(o);
        }
        if ((tid & 31) == 0) {
#pragma unroll
            for (int k = 0; k < 3; k++) wp[(tid >> 5) * 3 + k] = sum[k];
        }
        if (tid >= 32) {
            bar_arrive1(THREADS);
            return;
        }
        bar_wait1(THREADS);
#pragma unroll
        for (int k = 0; k < 3; k++) sum[k] = tid < NW ? wp[tid * 3 + k] : RowAcc<T>{};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int k = 0; k < 3; k++) sum[k].add_xor(o);
        }
        (void)sync;
#else
        // host emulation: each warp's partial is gathered in lane order
        for (int lane = 0; lane < 32; lane++) {
            if ((tid & 31) == lane) {
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    if (lane == 0) wp[(tid >> 5) * 3 + k] = sum[k];
                    else wp[(tid >> 5) * 3 + k].add(sum[k]);
                }
            }
            sync();
        }
        if (tid == 0) {
            RowAcc<T> t[3] = {wp[0], wp[1], wp[2]};
            for (int w = 1; w < NW; w++) {
#pragma unroll
                for (int k = 0; k < 3; k++) t[k].add(wp[w * 3 + k]);
            }
#pragma unroll
            for (int k = 0; k < 3; k++) sum[k] = t[k];
        }
#endif
    }

    // exp(L(k) h) at (kx, ky index iy): L = -(1 - k^2)^2 - alpha (lin_func,
    // ActFlow_V3-2.cu:1030) or -alpha - g0 k^2 - g2 k^4, evaluated in T.
    static AF_HD T lin_at(const StepArgs<T> &a, T kxv, int iy, T h)
    {
        T kyv = a.kyt[iy];
        T k2 = kyv * kyv + kxv * kxv;
        T Lk = a.form == 0 ? -(1 - k2) * (1 - k2) - a.alpha : -a.alpha - a.g0 * k2 - a.g2 * k2 * k2;
        return expT(Lk * h);
    }
};

}  // namespace af
