// Host-side set-up of one simulation: twiddle and wavenumber tables and the
// scalar kernel arguments.  Shared by the C ABI (actflow_api.cu) and the test
// suite's CPU execution of the kernel bodies, so both run identical set-up.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

#include "actflow.h"
#include "kernels.h"

namespace af {

// Reference dealias radius: (Nxh-1)*(Nxh-1)*Ny*Ny/4 in 32-bit int arithmetic
// (ActFlow_V3-2.cu:911); the products wrap modulo 2^32 on the GPU.
inline int reference_rsq(int nx, int ny)
{
    int nxh = nx / 2 + 1;
    uint32_t r = (uint32_t)(nxh - 1) * (uint32_t)(nxh - 1);
    r *= (uint32_t)ny;
    r *= (uint32_t)ny;
    return (int32_t)r / 4;
}

template <typename T>
struct HostTables {
    int nxh = 0, nt = 0;
    std::vector<cpx<T>> twx, twy;   // exp(-2 pi i m / N)
    std::vector<T> kx, ky;          // kx padded to nt * W entries
};

// Fill the tables and every scalar field of `a` (pointers are left alone).
// dt factors of the mean-flow stage updates, in double from dt as T: the same
// values the column pass would get from its own divisions.
template <typename T>
void set_mean_flow_coeffs(StepArgs<T> &a)
{
    const double dd = (double)a.dt;
    a.mf_d2 = dd / 2;
    a.mf_d6 = dd / 6;
    a.mf_d6l = dd / 6 * a.lin_v;
    a.mf_d3l2 = dd / 3 * a.lin2_v;
}

template <typename T>
void host_setup(const am_params &p, HostTables<T> &t, StepArgs<T> &a, int ecap)
{
    const int nx = p.nx, ny = p.ny;
    const int W = Tile<T>::W;
    t.nxh = nx / 2 + 1;
    t.nt = (t.nxh + W - 1) / W;
    // Twiddles, computed in double and rounded to T.
    t.twx.resize(nx);
    t.twy.resize(ny);
    for (int m = 0; m < nx; m++) {
        double ang = -2.0 * M_PI * (double)m / nx;
        t.twx[m] = mk((T)std::cos(ang), (T)std::sin(ang));
    }
    for (int m = 0; m < ny; m++) {
        double ang = -2.0 * M_PI * (double)m / ny;
        t.twy[m] = mk((T)std::cos(ang), (T)std::sin(ang));
    }
    // Wavenumbers 2 pi / L * n (wavenumber_func, ActFlow_V3-2.cu:1329-1349):
    // the box length is held in T (the reference parses it into a float), the
    // product is formed in double and rounded to T.  Rows are in FFT order.
    t.kx.assign((size_t)t.nt * W, (T)0);
    t.ky.resize(ny);
    const double lx = (double)(T)p.lx, ly = (double)(T)p.ly;
    for (int i = 0; i < t.nxh; i++) t.kx[i] = (T)(2.0 * M_PI / lx * i);
    for (int i = 0; i < ny; i++) t.ky[i] = (T)(2.0 * M_PI / ly * (i < ny / 2 + 1 ? i : i - ny));

    a.nx = nx;
    a.ny = ny;
    a.nxh = t.nxh;
    a.nt = t.nt;
    a.kxp = t.nxh - 1;
    a.ntp = t.nt;
    a.ecap = ecap;
    // FFT normalisation folded into lambda and beta in T, as the reference does
    // (ActFlow_V3-2.cu:434-436): lambda / N^2, beta / N^3.
    const double nd = (double)nx * (double)ny;
    if constexpr (std::is_same_v<T, df>) {
        // double-float: formed in double and split (host code does no
        // double-float arithmetic)
        a.lam_s = T(p.lambda / (nd * nd));
        a.beta_s = T(p.beta / (nd * nd * nd));
    } else {
        const T fnorm = (T)(nx * ny);
        a.lam_s = (T)p.lambda / (fnorm * fnorm);
        a.beta_s = (T)p.beta / (fnorm * fnorm * fnorm);
    }
    a.beta_sd = p.beta / (nd * nd * nd);
    a.dt = (T)p.dt;
    a.alpha = (T)p.alpha;
    a.g0 = (T)p.gamma0;
    a.g2 = (T)p.gamma2;
    a.form = p.form;
    a.dealias = p.dealias;
    a.rsq = reference_rsq(nx, ny);
    // Mean-flow integrating factors exp(L(0) dt), exp(L(0) dt / 2), in double
    // (the reference evaluates them in float, ActFlow_V3-2.cu:704-705).
    const double L0 = p.form == AM_FORM_REFERENCE ? -(1.0 + p.alpha) : -p.alpha;
    a.lin_v = std::exp(L0 * p.dt);
    a.lin2_v = std::exp(L0 * p.dt / 2);
    set_mean_flow_coeffs<T>(a);
    a.inv_2n3 = 1.0 / (2.0 * nd * nd * nd);
    a.mode = 0;
}

// Integrating factors: precomputed in double (a table read by the column
// pass) or evaluated per value in the state precision, as lin_func does.
// AM_IF_AUTO takes the table except for FP32 with the reference's mask (the
// parity mode, where the reference's own float exponentials are reproduced).
inline bool use_if_table(const am_params &p)
{
    if (p.if_factors == AM_IF_DOUBLE) return true;
    if (p.if_factors == AM_IF_FLOAT) return false;
    return !(p.precision == AM_FP32 && p.dealias == AM_DEALIAS_REFERENCE);
}

// Table coefficients: wavenumber steps 2 pi / L and the operator in double
// (the oracle's precision-form restatement uses the same expressions).
inline LinCoef lin_coef(const am_params &p)
{
    LinCoef c;
    c.kxs = 2.0 * M_PI / p.lx;
    c.kys = 2.0 * M_PI / p.ly;
    c.dt = p.dt;
    c.alpha = p.alpha;
    c.g0 = p.gamma0;
    c.g2 = p.gamma2;
    c.form = p.form;
    return c;
}

// Pruned transforms.  Under the 1/2 rule every nonlinear term vanishes outside
// the ellipse (kx/(Nx/2))^2 + (ky/(Ny/2))^2 <= 1/4, and the integrating factor
// maps zero to zero, so a state that is zero outside the ellipse stays zero
// there.  The stage fields then carry no data for kx > Nx/4: the column pass
// skips those tiles and the row pass neither loads nor stores them.  The results
// are those of the full transforms (the skipped entries are exact zeros).
// Per-run side buffer: the row sums (3 * Ny values) followed by the two
// halves of the kx = 0 column's w_new (2 * Ny complex), sized for double so
// one layout serves both precisions.
inline size_t side_bytes(int ny) { return (size_t)ny * (3 * sizeof(double) + 2 * 2 * sizeof(double)); }
template <typename T>
void set_side(StepArgs<T> &a, void *base, int ny)
{
    a.rowp = reinterpret_cast<T *>(base);
    a.hcol = reinterpret_cast<cpx<T> *>(static_cast<unsigned char *>(base) + (size_t)ny * 3 * sizeof(double));
}

template <typename T>
void set_pruning(StepArgs<T> &a, bool on)
{
    const int W = Tile<T>::W;
    if (on) {
        a.kxp = a.nx / 4;
        a.ntp = a.kxp / W + 1;
    } else {
        a.kxp = a.nxh - 1;
        a.ntp = a.nt;
    }
}

// True if the half-plane state w ([ny][nxh] complex, interleaved) is zero at
// every mode the 1/2 rule removes.
// The kept modes of a row form a prefix ix <= lim(iy) (mask_at's condition is
// monotone in ix), so each row's limit is found once and only the entries past
// it are tested.
// The entries past the limit are tested as bit patterns with each
// component's sign bit cleared (zero for +0 and -0 only, as x != 0), OR-ed
// over the row: a branch-free loop the compiler vectorises.  W is the word of
// one real component (32 bits for float and for each half of a double-float,
// 64 for double), per_cpx the words per complex value.  (The C ABI's
// set_state does this check on the device, in the tile kernel.)
template <typename W>
bool inside_half_mask_bits(const void *w, int per_cpx, int nx, int ny)
{
    constexpr W MAG = ~(W(1) << (8 * sizeof(W) - 1));
    const unsigned char *base = static_cast<const unsigned char *>(w);
    const int nxh = nx / 2 + 1;
    int lim = nxh - 1;   // kept ix of the row: 0..lim (lim = -1: none)
    for (int iy = 0; iy < ny; iy++) {
        while (lim >= 0 && !mask_at(1, 0, nx, ny, lim, iy)) lim--;
        while (lim + 1 < nxh && mask_at(1, 0, nx, ny, lim + 1, iy)) lim++;
        const unsigned char *row = base + (size_t)iy * nxh * per_cpx * sizeof(W);
        W acc = 0;
        for (int k = per_cpx * (lim + 1); k < per_cpx * nxh; k++) {
            W b;
            std::memcpy(&b, row + (size_t)k * sizeof(W), sizeof(W));
            acc |= b & MAG;
        }
        if (acc != 0) return false;
    }
    return true;
}
template <typename T>
bool state_inside_half_mask(const T *w, int nx, int ny)
{
    if constexpr (std::is_same_v<T, double>) return inside_half_mask_bits<uint64_t>(w, 2, nx, ny);
    else return inside_half_mask_bits<uint32_t>(w, 2 * (int)(sizeof(T) / 4), nx, ny);   // float, double-float
}

}  // namespace af
