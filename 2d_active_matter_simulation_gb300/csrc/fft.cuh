// Shared-memory Stockham FFT building blocks for the actflow step kernels.
//
// The same source compiles as CUDA device code (nvcc, sm_103a) and as plain C++
// (g++), so the test suite can execute the kernels' per-thread logic on the CPU
// with real threads and barriers.  Only the qualifier macros differ.
//
// Conventions
//  * cpx<T>: complex number {x = real, y = imaginary}, T = float, double or
//    df (double-float, dfloat.cuh).
//  * A length-L transform is computed by TPC = L/R threads; thread j holds the
//    elements j + r*TPC (r = 0..R-1) in registers on entry and on exit
//    ("cyclic distribution").  The first pass may use a smaller radix R1 (each
//    thread then runs R/R1 butterflies); every later pass has radix R.
//  * Pass with sub-transform size Ns (Stockham autosort, decimation in time,
//    as in Govindaraju et al., "High performance discrete Fourier transforms on
//    graphics processors", SC 2008): thread j reads x[j + r*TPC], multiplies by
//    W_{Ns R}^{r (j mod Ns)}, runs an R-point DFT and writes y[(j/Ns) Ns R +
//    (j mod Ns) + r Ns].  The last pass keeps its outputs in registers, which
//    for Ns = L/R are exactly y[j + r*TPC].
//  * Transforms are unnormalised; SIGN = -1 forward, +1 inverse.
#pragma once

#include <type_traits>

#include "dfloat.cuh"

#ifdef __CUDACC__
#define AF_HD __host__ __device__ __forceinline__
#define AF_HDC __host__ __device__
#define AF_DEV __device__ __forceinline__
#else
#include <math.h>

#include <cmath>
#define AF_HD inline
#define AF_HDC
#define AF_DEV inline
#endif

namespace af {

template <typename T>
struct alignas(2 * sizeof(T)) cpx {
    T x, y;
};

template <typename T>
AF_HD cpx<T> mk(T a, T b)
{
    cpx<T> r;
    r.x = a;
    r.y = b;
    return r;
}
template <typename T>
AF_HD cpx<T> operator+(cpx<T> a, cpx<T> b) { return mk(a.x + b.x, a.y + b.y); }
template <typename T>
AF_HD cpx<T> operator-(cpx<T> a, cpx<T> b) { return mk(a.x - b.x, a.y - b.y); }
// FP32 complex addition and subtraction on Blackwell's packed FP32x2 pipe:
// one instruction per complex value instead of two.  Both halves round as the
// scalar operations do (a - b is formed as fma(b, -1, a), whose product is
// exact), so results are bit-identical to the scalar forms.
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
template <>
AF_HD cpx<float> operator+(cpx<float> a, cpx<float> b)
{
    const float2 r = __fadd2_rn(make_float2(a.x, a.y), make_float2(b.x, b.y));
    return mk(r.x, r.y);
}
template <>
AF_HD cpx<float> operator-(cpx<float> a, cpx<float> b)
{
    const float2 r = __ffma2_rn(make_float2(b.x, b.y), make_float2(-1.0f, -1.0f), make_float2(a.x, a.y));
    return mk(r.x, r.y);
}
#endif
template <typename T>
AF_HD cpx<T> cmul(cpx<T> a, cpx<T> b) { return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// a * conj(b)
template <typename T>
AF_HD cpx<T> cmulc(cpx<T> a, cpx<T> b) { return mk(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
// FP32 complex products on the packed FP32x2 pipe: a product of both halves,
// then a fused multiply-add of both halves -- two roundings per component, as
// the scalar product-then-fma.
template <>
AF_HD cpx<float> cmul(cpx<float> a, cpx<float> b)
{
    const float2 t = __fmul2_rn(make_float2(a.x, a.x), make_float2(b.x, b.y));
    const float2 r = __ffma2_rn(make_float2(a.y, a.y), make_float2(-b.y, b.x), t);
    return mk(r.x, r.y);
}
template <>
AF_HD cpx<float> cmulc(cpx<float> a, cpx<float> b)
{
    const float2 t = __fmul2_rn(make_float2(a.x, a.y), make_float2(b.x, b.x));
    const float2 r = __ffma2_rn(make_float2(a.y, a.x), make_float2(b.y, -b.y), t);
    return mk(r.x, r.y);
}
#endif
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
// Double-float complex arithmetic on the packed FP32x2 pipe: the real and
// imaginary parts go through identical operation sequences, run side by side
// (df2, dfloat.cuh) -- half the instructions, bit-identical results to the
// scalar double-float forms (a - b is a + (-b) there, and negations are exact).
AF_HD cpx<df> df2_cpx(df2 v) { return mk(df2_first(v), df2_second(v)); }
template <>
AF_HD cpx<df> operator+(cpx<df> a, cpx<df> b) { return df2_cpx(df2_add(df2_of(a.x, a.y), df2_of(b.x, b.y))); }
template <>
AF_HD cpx<df> operator-(cpx<df> a, cpx<df> b) { return df2_cpx(df2_add(df2_of(a.x, a.y), df2_of(-b.x, -b.y))); }
template <>
AF_HD cpx<df> cmul(cpx<df> a, cpx<df> b)
{
    const df2 t = df2_mul(df2_of(a.x, a.x), df2_of(b.x, b.y));
    const df2 u = df2_mul(df2_of(a.y, a.y), df2_of(-b.y, b.x));
    return df2_cpx(df2_add(t, u));
}
template <>
AF_HD cpx<df> cmulc(cpx<df> a, cpx<df> b)
{
    const df2 t = df2_mul(df2_of(a.x, a.y), df2_of(b.x, b.x));
    const df2 u = df2_mul(df2_of(a.y, a.x), df2_of(b.y, -b.y));
    return df2_cpx(df2_add(t, u));
}
#endif
template <typename T>
AF_HD cpx<T> conj(cpx<T> a) { return mk(a.x, -a.y); }
template <typename T>
AF_HD cpx<T> scale(cpx<T> a, T s) { return mk(a.x * s, a.y * s); }
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
template <>
AF_HD cpx<float> scale(cpx<float> a, float s)
{
    const float2 r = __fmul2_rn(make_float2(a.x, a.y), make_float2(s, s));
    return mk(r.x, r.y);
}
template <>
AF_HD cpx<df> scale(cpx<df> a, df s) { return df2_cpx(df2_mul(df2_of(a.x, a.y), df2_of(s, s))); }
#endif

// a + s b, component by component (s = (sx, sy), used with s = +-1, where the
// products are exact); FP32 on Blackwell: one packed fused multiply-add.
template <typename T>
AF_HD cpx<T> cfma(cpx<T> s, cpx<T> b, cpx<T> a) { return mk(a.x + s.x * b.x, a.y + s.y * b.y); }
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
template <>
AF_HD cpx<float> cfma(cpx<float> s, cpx<float> b, cpx<float> a)
{
    const float2 r = __ffma2_rn(make_float2(s.x, s.y), make_float2(b.x, b.y), make_float2(a.x, a.y));
    return mk(r.x, r.y);
}
#endif

// w + f n (double-float: as complex operations on the packed pipe).
template <typename T>
AF_HD cpx<T> axpy(cpx<T> w, T f, cpx<T> n)
{
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
    if constexpr (std::is_same_v<T, df>) return w + scale(n, f);
#endif
    return mk(w.x + f * n.x, w.y + f * n.y);
}

// Multiply by exp(SIGN * 2 pi i Q / R) for compile-time Q, R (R <= 32).
// Multiples of pi/2 are exact sign swaps; the remaining angles are multiples
// of pi/16, whose cosines are the constants below.
template <int Q, int R, int SIGN, typename T>
AF_HD cpx<T> rot(cpx<T> a)
{
    constexpr int N32 = (32 / R) * Q;          // angle in units of 2 pi / 32
    constexpr int q = ((N32 % 32) + 32) % 32;
    if constexpr (q == 0) {
        return a;
    } else if constexpr (q == 8) {             // pi/2: multiply by SIGN * i
        return SIGN > 0 ? mk(-a.y, a.x) : mk(a.y, -a.x);
    } else if constexpr (q == 16) {
        return mk(-a.x, -a.y);
    } else if constexpr (q == 24) {
        return SIGN > 0 ? mk(a.y, -a.x) : mk(-a.y, a.x);
    } else {
        // cos(2 pi k / 32), k = 0..8
        constexpr double C[9] = {1.0,
                                 0.98078528040323044913,
                                 0.92387953251128675613,
                                 0.83146961230254523708,
                                 0.70710678118654752440,
                                 0.55557023301960222474,
                                 0.38268343236508977173,
                                 0.19509032201612826785,
                                 0.0};
        constexpr int qq = q % 8;              // offset inside the quadrant
        constexpr int quad = q / 8;
        constexpr double c0 = C[qq], s0 = C[8 - qq];
        constexpr double cs = quad == 0 ? c0 : quad == 1 ? -s0 : quad == 2 ? -c0 : s0;
        constexpr double sn = quad == 0 ? s0 : quad == 1 ? c0 : quad == 2 ? -s0 : -c0;
        const T c = (T)cs, s = (T)(SIGN * sn);
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
        if constexpr (sizeof(T) == 4) {   // packed FP32x2: product, then fma (as cmul)
            const float2 t = __fmul2_rn(make_float2(a.x, a.x), make_float2(c, s));
            const float2 r = __ffma2_rn(make_float2(a.y, a.y), make_float2(-s, c), t);
            return mk(r.x, r.y);
        }
        if constexpr (std::is_same_v<T, df>) return cmul(a, mk(c, s));   // packed double-float
#endif
        return mk(a.x * c - a.y * s, a.x * s + a.y * c);
    }
}

// Calls f(std::integral_constant<int, I>) for I = I0 .. N-1 (compile-time loop).
template <int I0, int N, class Fn>
AF_HD void static_for(Fn &&f)
{
    if constexpr (I0 < N) {
        f(std::integral_constant<int, I0>{});
        static_for<I0 + 1, N>(f);
    }
}

// In-register R-point DFT, natural order in and out (radix-2 decimation in
// time, fully unrolled at compile time).
template <int R, int SIGN, typename T>
struct DFT {
    static AF_HD void run(cpx<T> *v)
    {
        if constexpr (R == 1) {
            return;
        } else if constexpr (R == 2) {
            cpx<T> a = v[0], b = v[1];
            v[0] = a + b;
            v[1] = a - b;
        } else {
            cpx<T> e[R / 2], o[R / 2];
#pragma unroll
            for (int i = 0; i < R / 2; i++) {
                e[i] = v[2 * i];
                o[i] = v[2 * i + 1];
            }
            DFT<R / 2, SIGN, T>::run(e);
            DFT<R / 2, SIGN, T>::run(o);
            combine<0>(v, e, o);
        }
    }
    template <int Q>
    static AF_HD void combine(cpx<T> *v, const cpx<T> *e, const cpx<T> *o)
    {
        if constexpr (Q < R / 2) {
            cpx<T> t = rot<Q, R, SIGN, T>(o[Q]);
            v[Q] = e[Q] + t;
            v[Q + R / 2] = e[Q] - t;
            combine<Q + 1>(v, e, o);
        }
    }
};

// Shared-memory exchange buffer for W interleaved transforms (W columns of a
// tile, or W = 1 for a single row).  Complex values are stored whole (one
// 8- or 16-byte access each); element idx of transform c sits at slot
// SWZ(idx) * W + c.  The index maps were chosen by simulating the bank pattern of
// every pass of the transforms that use them (vector accesses are served per
// half- or quarter-warp):
//   SWZ 0: idx + idx/8          column passes (W = 4 FP32, W = 2 FP64)
//   SWZ 1: idx ^ ((idx/16) % 16) row passes, FP32 (a permutation: no padding)
//   SWZ 2: idx + idx/4          row passes, FP64
//   SWZ 5: per exchange, keyed on the write stride NS of the exchange: NS = 2
//          idx ^ ((idx/8) % 16), NS = 4 idx ^ (bits 5-6 of idx moved to bits
//          2-3), NS = 8 idx ^ (bit 6 of idx moved to bit 3), otherwise as
//          SWZ 1 -- row passes, FP32: conflict-free for every exchange of the
//          transforms of 16 to 2048 points (SWZ 1 alone: 1.25x the
//          conflict-free wavefronts at 1024 and 256 points, 1.17x at 2048;
//          its NS = 4 and NS = 8 writes are 2-way conflicts); put/get use
//          the SWZ 1 map
template <typename T, int W, int SWZ>
struct XBuf {
    cpx<T> *d;
    // additive pads i + (i >> SH): pad(b + r s) = pad(b) + r (s + s >> SH)
    // whenever s is a multiple of 2^SH, so strided accesses need one index
    // computation per pass (see at()).
    static constexpr int SH = SWZ == 0 ? 3 : SWZ == 2 ? 2 : SWZ == 3 ? 4 : SWZ == 4 ? 5 : 0;
    AF_HDC static constexpr int pad(int i)
    {
        if constexpr (SWZ == 0) return i + (i >> 3);
        else if constexpr (SWZ == 1 || SWZ == 5) return i ^ ((i >> 4) & 15);
        else if constexpr (SWZ == 2) return i + (i >> 2);
        else if constexpr (SWZ == 3) return i + (i >> 4);
        else return i + (i >> 5);
    }
    // Slot of element base + r * STRIDE for transform c, in the exchange whose
    // writes have stride NSX (SWZ 5 picks its map by it; others ignore it).
    template <int STRIDE, int NSX = STRIDE>
    AF_HD int at(int base, int r, int c) const
    {
        if constexpr (SWZ == 5 && NSX == 2) {
            const int i = base + r * STRIDE;
            return (i ^ ((i >> 3) & 15)) * W + c;
        } else if constexpr (SWZ == 5 && NSX == 4) {
            const int i = base + r * STRIDE;
            return (i ^ ((i >> 3) & 12)) * W + c;
        } else if constexpr (SWZ == 5 && NSX == 8) {
            const int i = base + r * STRIDE;
            return (i ^ ((i >> 3) & 8)) * W + c;
        } else if constexpr (SWZ != 1 && SWZ != 5 && (STRIDE % (1 << SH)) == 0) {
            return (pad(base) + r * (STRIDE + (STRIDE >> SH))) * W + c;
        } else {
            return pad(base + r * STRIDE) * W + c;
        }
    }
    // slots needed for L elements
    AF_HDC static constexpr int slots(int L)
    {
        if constexpr (SWZ == 1 || SWZ == 5) return (L < 16 ? 16 : L) * W;
        else return pad(L - 1) * W + W;
    }
    AF_HD void put(int idx, int c, cpx<T> v) const { d[pad(idx) * W + c] = v; }
    AF_HD cpx<T> get(int idx, int c) const { return d[pad(idx) * W + c]; }
};

// Twiddle source: tw[m * STRIDE] = exp(-2 pi i m / L) for m < L.
AF_HD cpx<float> ldtw(const cpx<float> *tw, int idx)
{
#ifdef __CUDA_ARCH__
    float2 v = __ldg(reinterpret_cast<const float2 *>(tw) + idx);
    return mk(v.x, v.y);
#else
    return tw[idx];
#endif
}
AF_HD cpx<double> ldtw(const cpx<double> *tw, int idx)
{
#ifdef __CUDA_ARCH__
    double2 v = __ldg(reinterpret_cast<const double2 *>(tw) + idx);
    return mk(v.x, v.y);
#else
    return tw[idx];
#endif
}
AF_HD cpx<df> ldtw(const cpx<df> *tw, int idx)
{
#ifdef __CUDA_ARCH__
    float4 v = __ldg(reinterpret_cast<const float4 *>(tw) + idx);
    return mk(df(v.x, v.y), df(v.z, v.w));
#else
    return tw[idx];
#endif
}

// Length-L (L = 2^LOGL) block FFT on data distributed cyclically over TPC =
// L/R threads.  `sync` is the block barrier (called identically by every
// thread of the block).  tw must hold exp(-2 pi i m / (L * TWS)) at index m for
// m < L * TWS; the transform uses every TWS-th entry.
// Twiddle powers w[r] = W^{r k} (r = 1..R-1) for one pass, from the table
// entry at r * step.  FP32: the powers 1, 2, 4, 8 are loaded and the others
// formed by at most three complex products (error a few ulp); FP64 and
// double-float (8-byte reals): all loaded.
template <int R, typename T>
AF_HD void twiddles(cpx<T> *w, const cpx<T> *tw, int step)
{
    if constexpr (sizeof(T) == 4 && R <= 8 && R > 2) {
        // radix <= 8, FP32: one table load; W^2k, W^4k by squaring and the
        // rest by products (at most three roundings deep, a few ulp).
        w[1] = ldtw(tw, step);
        w[2] = cmul(w[1], w[1]);
        w[3] = cmul(w[2], w[1]);
        if constexpr (R == 8) {
            w[4] = cmul(w[2], w[2]);
            w[5] = cmul(w[4], w[1]);
            w[6] = cmul(w[4], w[2]);
            w[7] = cmul(w[4], w[3]);
        }
    } else if constexpr (sizeof(T) == 4 && R == 16) {
        // radix 16, FP32: W^k and W^4k loaded, the rest by products (at most
        // four roundings deep)
        w[1] = ldtw(tw, step);
        w[4] = ldtw(tw, 4 * step);
        w[2] = cmul(w[1], w[1]);
        w[3] = cmul(w[2], w[1]);
        w[5] = cmul(w[4], w[1]);
        w[6] = cmul(w[4], w[2]);
        w[7] = cmul(w[4], w[3]);
        w[8] = cmul(w[4], w[4]);
#pragma unroll
        for (int r = 9; r < 16; r++) w[r] = cmul(w[8], w[r - 8]);
    } else if constexpr (sizeof(T) == 8 || R <= 2) {
#pragma unroll
        for (int r = 1; r < R; r++) w[r] = ldtw(tw, r * step);
    } else {
        w[1] = ldtw(tw, step);
        w[2] = ldtw(tw, 2 * step);
        w[3] = cmul(w[2], w[1]);
        if constexpr (R >= 8) {
            w[4] = ldtw(tw, 4 * step);
            w[5] = cmul(w[4], w[1]);
            w[6] = cmul(w[4], w[2]);
            w[7] = cmul(w[4], w[3]);
        }
        if constexpr (R >= 16) {
            w[8] = ldtw(tw, 8 * step);
#pragma unroll
            for (int r = 9; r < 16; r++) w[r] = cmul(w[8], w[r - 8]);
        }
        if constexpr (R >= 32) {
            w[16] = ldtw(tw, 16 * step);
#pragma unroll
            for (int r = 17; r < 32; r++) w[r] = cmul(w[16], w[r - 16]);
        }
    }
}

template <typename T, int LOGL, int LOGR_MAX, int SIGN>
struct BlockFFT {
    static constexpr int LOGR = LOGR_MAX < LOGL ? LOGR_MAX : LOGL;
    static constexpr int R = 1 << LOGR;
    static constexpr int L = 1 << LOGL;
    static constexpr int TPC = L / R;
    static constexpr int LOGR1 = LOGL % LOGR;
    static constexpr int R1 = 1 << LOGR1;          // first-pass radix (1: none)
    static constexpr int NPASS = (LOGL - LOGR1) / LOGR;
    static constexpr int NEXCH = NPASS - 1 + (LOGR1 > 0 ? 1 : 0);   // shared-memory exchanges

    // Exchanges alternate between two buffers b0, b1 (b1 may equal b0): with
    // two buffers one barrier per exchange suffices, because the barrier that
    // publishes exchange e also orders every read of exchange e-1 before the
    // writes of exchange e+1.  One barrier at entry separates this transform
    // from earlier users of the buffers.
    template <class Buf, class Sync>
    static AF_HD void run(cpx<T> (&v)[R], int j, int c, const Buf &b0, const Buf &b1, const cpx<T> *tw, int TWS,
                          Sync &&sync)
    {
        if constexpr (NEXCH > 0) sync();
        run_passes<0>(v, j, c, b0, b1, tw, TWS, sync);
    }
    template <class Buf, class Sync>
    static AF_HD void run(cpx<T> (&v)[R], int j, int c, const Buf &buf, const cpx<T> *tw, int TWS, Sync &&sync)
    {
        if constexpr (NEXCH > 0) sync();
        run_passes<1>(v, j, c, buf, buf, tw, TWS, sync);
    }

    template <int SINGLE, class Buf, class Sync>
    static AF_HD void run_passes(cpx<T> (&v)[R], int j, int c, const Buf &b0, const Buf &b1, const cpx<T> *tw,
                                 int TWS, Sync &&sync)
    {
        int e = 0;   // exchange counter: buffer e % 2
        if constexpr (LOGR1 > 0) {
            constexpr int G = R / R1;
#pragma unroll
            for (int q = 0; q < G; q++) {
                cpx<T> u[R1];
#pragma unroll
                for (int r1 = 0; r1 < R1; r1++) u[r1] = v[q + G * r1];
                DFT<R1, SIGN, T>::run(u);
#pragma unroll
                for (int r1 = 0; r1 < R1; r1++) v[q + G * r1] = u[r1];
            }
            const Buf &b = b0;
#pragma unroll
            for (int q = 0; q < G; q++) {
                const int base = (j + q * TPC) * R1;
#pragma unroll
                for (int r1 = 0; r1 < R1; r1++) b.d[b.template at<1>(base, r1, c)] = v[q + G * r1];
            }
            sync();
            e = 1;
        }
        pass<0, LOGR1 == 0, SINGLE>(v, j, c, b0, b1, tw, TWS, sync, e);
    }

    // Radix-R pass number P (sub-transform size NS = R1 * R^P).
    template <int P, bool FROM_REGS, int SINGLE, class Buf, class Sync>
    static AF_HD void pass(cpx<T> (&v)[R], int j, int c, const Buf &b0, const Buf &b1, const cpx<T> *tw, int TWS,
                           Sync &&sync, int e)
    {
        if constexpr (P < NPASS) {
            constexpr int NS = R1 * ipow(R, P);
            if constexpr (!FROM_REGS) {
                const Buf &b = (SINGLE || (e & 1) == 1) ? b0 : b1;   // buffer written by exchange e-1
#pragma unroll
                for (int r = 0; r < R; r++) v[r] = b.d[b.template at<TPC, (P == 0 ? 1 : NS / R)>(j, r, c)];
            }
            if constexpr (NS > 1) {
                const int k = j & (NS - 1);
                const int step = (L / (NS * R)) * k * TWS;   // twiddle index of W^{k}
                if constexpr (R >= 32) {
                    // radix 32: each twiddle is read from the (L1-resident) table
                    // right before use, so no twiddle array is held in registers
#pragma unroll
                    for (int r = 1; r < R; r++) {
                        const cpx<T> w = ldtw(tw, r * step);
                        v[r] = SIGN < 0 ? cmul(v[r], w) : cmulc(v[r], w);
                    }
                } else {
                    cpx<T> w[R];
                    twiddles<R>(w, tw, step);
#pragma unroll
                    for (int r = 1; r < R; r++) v[r] = SIGN < 0 ? cmul(v[r], w[r]) : cmulc(v[r], w[r]);
                }
            }
            DFT<R, SIGN, T>::run(v);
            if constexpr (P < NPASS - 1) {
                const Buf &b = (SINGLE || (e & 1) == 0) ? b0 : b1;
                const int k = j & (NS - 1);
                const int base = (j - k) * R + k;
                if (SINGLE && e > 0) sync();   // one buffer: earlier reads must finish
#pragma unroll
                for (int r = 0; r < R; r++) b.d[b.template at<NS, NS>(base, r, c)] = v[r];
                sync();
                pass<P + 1, false, SINGLE>(v, j, c, b0, b1, tw, TWS, sync, e + 1);
            }
        }
    }

    static constexpr int ipow(int b, int p) { return p == 0 ? 1 : b * ipow(b, p - 1); }

    // The same transform with one buffer (as run(v, j, c, buf, ...)), in a
    // compact form: the radix-R passes are a loop that is not unrolled (one
    // pass body in the code instead of NPASS), and the inverse transform is
    // the forward one between conjugations (conj F(conj x)), so both
    // directions share that body's shape.  For arithmetic whose operations
    // expand to many instructions (double-float), where the unrolled
    // transforms outgrow the instruction caches.
    template <class Buf, class Sync>
    static AF_HD void run_compact(cpx<T> (&v)[R], int j, int c, const Buf &b, const cpx<T> *tw, int TWS,
                                  Sync &&sync)
    {
        if constexpr (SIGN > 0) {
#pragma unroll
            for (int r = 0; r < R; r++) v[r] = conj(v[r]);
        }
        if constexpr (NEXCH > 0) sync();
        bool in_buf = false;   // this pass's input is in the buffer (else in registers)
        if constexpr (LOGR1 > 0) {
            constexpr int G = R / R1;
#pragma unroll
            for (int q = 0; q < G; q++) {
                cpx<T> u[R1];
#pragma unroll
                for (int r1 = 0; r1 < R1; r1++) u[r1] = v[q + G * r1];
                DFT<R1, -1, T>::run(u);
                const int base = (j + q * TPC) * R1;
#pragma unroll
                for (int r1 = 0; r1 < R1; r1++) b.put(base + r1, c, u[r1]);
            }
            sync();
            in_buf = true;
        }
#pragma unroll 1
        for (int p = 0; p < NPASS; p++) {
            const int ns = R1 << (LOGR * p);   // sub-transform size of this pass
            if (in_buf) {
#pragma unroll
                for (int r = 0; r < R; r++) v[r] = b.get(j + r * TPC, c);
            }
            if (ns > 1) {
                const int k = j & (ns - 1);
                cpx<T> w[R];
                twiddles<R>(w, tw, (L / (ns * R)) * k * TWS);
#pragma unroll
                for (int r = 1; r < R; r++) v[r] = cmul(v[r], w[r]);
            }
            DFT<R, -1, T>::run(v);
            if (p < NPASS - 1) {
                const int k = j & (ns - 1);
                const int base = (j - k) * R + k;
                if (in_buf) sync();   // one buffer: this pass's reads must finish first
#pragma unroll
                for (int r = 0; r < R; r++) b.put(base + r * ns, c, v[r]);
                sync();
                in_buf = true;
            }
        }
        if constexpr (SIGN > 0) {
#pragma unroll
            for (int r = 0; r < R; r++) v[r] = conj(v[r]);
        }
    }

    // NF transforms of the same length and direction in lockstep: v[f] holds
    // transform f (cyclic distribution), b0[f] / b1[f] are its two exchange
    // buffers.  The twiddles of a pass are formed once for all NF transforms
    // and one barrier per exchange serves all of them, and the NF independent
    // DFTs per thread give the scheduler more work between shared-memory
    // accesses.  SINGLE = 1: b1 is ignored and each transform reuses b0[f] for
    // every exchange (one more barrier per exchange, half the shared memory).
    template <int NF, int SINGLE = 0, class Buf, class Sync>
    static AF_HD void run_multi(cpx<T> (&v)[NF][R], int j, int c, const Buf (&b0)[NF], const Buf (&b1)[NF],
                                const cpx<T> *tw, int TWS, Sync &&sync)
    {
        if constexpr (NEXCH > 0) sync();
        int e = 0;
        if constexpr (LOGR1 > 0) {
            constexpr int G = R / R1;
#pragma unroll
            for (int f = 0; f < NF; f++) {
#pragma unroll
                for (int q = 0; q < G; q++) {
                    cpx<T> u[R1];
#pragma unroll
                    for (int r1 = 0; r1 < R1; r1++) u[r1] = v[f][q + G * r1];
                    DFT<R1, SIGN, T>::run(u);
                    const int base = (j + q * TPC) * R1;
#pragma unroll
                    for (int r1 = 0; r1 < R1; r1++) b0[f].d[b0[f].template at<1>(base, r1, c)] = u[r1];
                }
            }
            sync();
            e = 1;
        }
        pass_multi<0, LOGR1 == 0, NF, SINGLE>(v, j, c, b0, b1, tw, TWS, sync, e);
    }

    template <int P, bool FROM_REGS, int NF, int SINGLE, class Buf, class Sync>
    static AF_HD void pass_multi(cpx<T> (&v)[NF][R], int j, int c, const Buf (&b0)[NF], const Buf (&b1)[NF],
                                 const cpx<T> *tw, int TWS, Sync &&sync, int e)
    {
        if constexpr (P < NPASS) {
            constexpr int NS = R1 * ipow(R, P);
            if constexpr (!FROM_REGS) {
#pragma unroll
                for (int f = 0; f < NF; f++) {
                    const Buf &b = (SINGLE || (e & 1) == 1) ? b0[f] : b1[f];   // written by exchange e-1
#pragma unroll
                    for (int r = 0; r < R; r++) v[f][r] = b.d[b.template at<TPC, (P == 0 ? 1 : NS / R)>(j, r, c)];
                }
            }
            if constexpr (NS > 1) {
                const int k = j & (NS - 1);
                const int step = (L / (NS * R)) * k * TWS;
                cpx<T> w[R];
                twiddles<R>(w, tw, step);
#pragma unroll
                for (int f = 0; f < NF; f++)
#pragma unroll
                    for (int r = 1; r < R; r++) v[f][r] = SIGN < 0 ? cmul(v[f][r], w[r]) : cmulc(v[f][r], w[r]);
            }
#pragma unroll
            for (int f = 0; f < NF; f++) DFT<R, SIGN, T>::run(v[f]);
            if constexpr (P < NPASS - 1) {
                const int k = j & (NS - 1);
                const int base = (j - k) * R + k;
                if (SINGLE && e > 0) sync();   // one buffer: earlier reads must finish
#pragma unroll
                for (int f = 0; f < NF; f++) {
                    const Buf &b = (SINGLE || (e & 1) == 0) ? b0[f] : b1[f];
#pragma unroll
                    for (int r = 0; r < R; r++) b.d[b.template at<NS, NS>(base, r, c)] = v[f][r];
                }
                sync();
                pass_multi<P + 1, false, NF, SINGLE>(v, j, c, b0, b1, tw, TWS, sync, e + 1);
            }
        }
    }
};

}  // namespace af
