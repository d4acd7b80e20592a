/*
 * actflow oracle: CPU restatement of the reference program's time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the tests, smoke()
 * and the CPU-baseline leg of bench.py call it to produce the expected results
 * and to time a CPU implementation of the step.  The product (the CUDA solver
 * behind include/actflow.h) never links, loads or calls it.
 *
 * Reference: ActFlow_V3-2.cu (DominikSuchla/2D_active_matter_simulation).  The
 * precision-generic core lives in oracle_core.h and is compiled twice: once in
 * float (the reference's own precision: cuComplex/float arrays, float exp,
 * ActFlow_V3-2.cu:449-495, 1030) and once in double (the FP64 oracle).
 *
 * Deviations from the reference, all deliberate:
 *  - the FFT is this file's own radix-2 transform (the reference calls cuFFT,
 *    a closed library), so FP32 results agree with the reference to rounding,
 *    not bit for bit;
 *  - the energy is accumulated in double (the reference sums in float on one
 *    host core, ActFlow_V3-2.cu:1118-1124).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int nx, ny;
    double lx, ly, dt;
    double lam, alpha, beta;
    double gamma0, gamma2;
    int form;    /* 0: reference operator -(1-k^2)^2 - alpha; 1: -alpha - g0 k^2 - g2 k^4 */
    int dealias; /* 0: reference mask (int32 arithmetic), 1: isotropic 1/2 rule, 2: none */
    int if_double; /* 0: integrating factors evaluated in REAL (lin_func); 1: in double from
                    * double wavenumbers and parameters, then rounded to REAL */
} orc_params;

/* Dealiasing mask value at half-plane index (ix, iy).
 *
 * Mode 0 restates cutoff_func (ActFlow_V3-2.cu:899-919) including its 32-bit
 * integer arithmetic: R_sq = (Nxh-1)*(Nxh-1)*Ny*Ny/4 is evaluated left to right
 * in int, which wraps modulo 2^32 on the GPU; the wrapped value is emulated
 * here with unsigned arithmetic, then divided by 4 with truncation toward zero.
 * Mode 1 keeps (ix/(Nx/2))^2 + (ky/(Ny/2))^2 <= 1/4, evaluated exactly in
 * 64-bit integers as 16 (ix^2 Ny^2 + ky^2 Nx^2) <= Nx^2 Ny^2, with ky the signed
 * row wavenumber index.  Mode 2 keeps every mode. */
int orc_mask_value(int nx, int ny, int mode, int ix, int iy)
{
    int nxh = nx / 2 + 1;
    if (mode == 0) {
        uint32_t r = (uint32_t)(nxh - 1) * (uint32_t)(nxh - 1);
        r *= (uint32_t)ny;
        r *= (uint32_t)ny;
        int32_t rsq = (int32_t)r / 4;
        if (ix * ix + iy * iy <= rsq) return 1;
        if (ix * ix + (ny - iy) * (ny - iy) <= rsq) return 1;
        return 0;
    }
    if (mode == 1) {
        int64_t ky = iy <= ny / 2 ? iy : iy - ny;
        int64_t X = ix, NX = nx, NY = ny;
        return 16 * (X * X * NY * NY + ky * ky * NX * NX) <= NX * NX * NY * NY;
    }
    return 1;
}

void orc_mask(int nx, int ny, int mode, float *out)
{
    int nxh = nx / 2 + 1;
    for (int iy = 0; iy < ny; iy++)
        for (int ix = 0; ix < nxh; ix++) out[(size_t)iy * nxh + ix] = (float)orc_mask_value(nx, ny, mode, ix, iy);
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

#define REAL float
#define SFX f32
#define EXPR expf
#include "oracle_core.h"
#undef REAL
#undef SFX
#undef EXPR

#define REAL double
#define SFX f64
#define EXPR exp
#include "oracle_core.h"
#undef REAL
#undef SFX
#undef EXPR
