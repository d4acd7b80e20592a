/*
 * Oracle core, instantiated once per precision by actflow_oracle.c with
 *   REAL  -- float or double
 *   SFX   -- name suffix (f32 / f64)
 *   EXPR  -- exp for REAL
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain CPU restatement of the reference
 * program's time step (ActFlow_V3-2.cu), used by the tests, by smoke() and by
 * the CPU-baseline leg of bench.py as the checker.  The product never calls it.
 *
 * It follows the reference's own sequence of operations: separate ux, uy and
 * omega inverse transforms, four separate forward transforms of the real-space
 * products, the odd integrating-factor RK stage formulas, the Hermitian repair
 * of the kx=0 column, the scaled mean velocity in the k=0 slot, and the folding
 * of the FFT normalisation into lambda and beta.  Each block cites the lines it
 * restates.
 */

#define CAT_(a, b) a##_##b
#define CAT(a, b) CAT_(a, b)
#define F(name) CAT(name, SFX)

typedef struct {
    REAL re, im;
} F(cplx);

/* ------------------------------------------------------------------ FFT --- */
/* Iterative radix-2 complex FFT, unnormalised; sign = -1 forward, +1 inverse.
 * Twiddles are computed in double and rounded to REAL.  Power-of-two lengths. */

typedef struct {
    int n, logn;
    F(cplx) * tw; /* exp(-2 pi i k / n), k < n/2 */
    int *rev;
} F(fftplan);

static int F(plan_init)(F(fftplan) * p, int n)
{
    int logn = 0;
    while ((1 << logn) < n) logn++;
    if ((1 << logn) != n) return -1;
    p->n = n;
    p->logn = logn;
    p->tw = (F(cplx) *)malloc(sizeof(F(cplx)) * (size_t)(n / 2 > 0 ? n / 2 : 1));
    p->rev = (int *)malloc(sizeof(int) * (size_t)n);
    for (int k = 0; k < n / 2; k++) {
        double a = -2.0 * M_PI * (double)k / (double)n;
        p->tw[k].re = (REAL)cos(a);
        p->tw[k].im = (REAL)sin(a);
    }
    for (int i = 0; i < n; i++) {
        int r = 0;
        for (int b = 0; b < logn; b++)
            if (i & (1 << b)) r |= 1 << (logn - 1 - b);
        p->rev[i] = r;
    }
    return 0;
}

static void F(plan_free)(F(fftplan) * p)
{
    free(p->tw);
    free(p->rev);
}

static void F(fft1d)(const F(fftplan) * p, F(cplx) * x, int sign)
{
    int n = p->n;
    for (int i = 0; i < n; i++) {
        int r = p->rev[i];
        if (r > i) {
            F(cplx) t = x[i];
            x[i] = x[r];
            x[r] = t;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1, step = n / len;
        for (int s = 0; s < n; s += len) {
            for (int k = 0; k < half; k++) {
                F(cplx) w = p->tw[k * step];
                if (sign > 0) w.im = -w.im;
                F(cplx) a = x[s + k], b = x[s + k + half];
                REAL br = b.re * w.re - b.im * w.im;
                REAL bi = b.re * w.im + b.im * w.re;
                x[s + k].re = a.re + br;
                x[s + k].im = a.im + bi;
                x[s + k + half].re = a.re - br;
                x[s + k + half].im = a.im - bi;
            }
        }
    }
}

typedef struct {
    int nx, ny, nxh;
    F(fftplan) px, py;
} F(plan2d);

static int F(plan2d_init)(F(plan2d) * p, int nx, int ny)
{
    p->nx = nx;
    p->ny = ny;
    p->nxh = nx / 2 + 1;
    if (F(plan_init)(&p->px, nx)) return -1;
    if (F(plan_init)(&p->py, ny)) return -1;
    return 0;
}

static void F(plan2d_free)(F(plan2d) * p)
{
    F(plan_free)(&p->px);
    F(plan_free)(&p->py);
}

/* 2-D R2C, unnormalised: real [ny][nx] -> half plane [ny][nxh]
 * (the transform the reference gets from cufftPlan2d(..., CUFFT_R2C),
 * ActFlow_V3-2.cu:507). */
static void F(rfft2)(const F(plan2d) * p, const REAL *in, F(cplx) * out)
{
    int nx = p->nx, ny = p->ny, nxh = p->nxh;
#pragma omp parallel
    {
        F(cplx) *buf = (F(cplx) *)malloc(sizeof(F(cplx)) * (size_t)(nx > ny ? nx : ny));
#pragma omp for schedule(static)
        for (int y = 0; y < ny; y++) {
            for (int x = 0; x < nx; x++) {
                buf[x].re = in[(size_t)y * nx + x];
                buf[x].im = 0;
            }
            F(fft1d)(&p->px, buf, -1);
            for (int k = 0; k < nxh; k++) out[(size_t)y * nxh + k] = buf[k];
        }
#pragma omp for schedule(static)
        for (int k = 0; k < nxh; k++) {
            for (int y = 0; y < ny; y++) buf[y] = out[(size_t)y * nxh + k];
            F(fft1d)(&p->py, buf, -1);
            for (int y = 0; y < ny; y++) out[(size_t)y * nxh + k] = buf[y];
        }
        free(buf);
    }
}

/* 2-D C2R, unnormalised: half plane [ny][nxh] -> real [ny][nx]
 * (cufftPlan2d(..., CUFFT_C2R), ActFlow_V3-2.cu:508).  Inverse transforms along
 * y first, then each row is extended by Hermitian symmetry; the imaginary parts
 * of the kx=0 and kx=nx/2 entries of each row are dropped, which is what a
 * half-plane C2R does with a spectrum that is not exactly Hermitian. */
static void F(irfft2)(const F(plan2d) * p, const F(cplx) * in, REAL *out)
{
    int nx = p->nx, ny = p->ny, nxh = p->nxh;
    F(cplx) *tmp = (F(cplx) *)malloc(sizeof(F(cplx)) * (size_t)ny * nxh);
#pragma omp parallel
    {
        F(cplx) *buf = (F(cplx) *)malloc(sizeof(F(cplx)) * (size_t)(nx > ny ? nx : ny));
#pragma omp for schedule(static)
        for (int k = 0; k < nxh; k++) {
            for (int y = 0; y < ny; y++) buf[y] = in[(size_t)y * nxh + k];
            F(fft1d)(&p->py, buf, +1);
            for (int y = 0; y < ny; y++) tmp[(size_t)y * nxh + k] = buf[y];
        }
#pragma omp for schedule(static)
        for (int y = 0; y < ny; y++) {
            const F(cplx) *row = tmp + (size_t)y * nxh;
            for (int k = 0; k < nxh; k++) buf[k] = row[k];
            buf[0].im = 0;
            if (nx % 2 == 0) buf[nx / 2].im = 0;
            for (int k = nxh; k < nx; k++) {
                buf[k].re = row[nx - k].re;
                buf[k].im = -row[nx - k].im;
            }
            F(fft1d)(&p->px, buf, +1);
            for (int x = 0; x < nx; x++) out[(size_t)y * nx + x] = buf[x].re;
        }
        free(buf);
    }
    free(tmp);
}

/* --------------------------------------------------------- the solver --- */

typedef struct {
    int nx, ny, nxh, size;
    REAL dt, lam, beta;        /* lam, beta already divided by N^2, N^3 */
    REAL lin_v, lin2_v;        /* mean-flow integrating factors */
    REAL *kx, *ky, *k2, *mask, *lin, *lin2;
    F(cplx) *w_old, *w_new, *w_appr, *nonl;
    F(cplx) *vx_c, *vy_c, *arr_c;   /* spectral work arrays */
    REAL *vx, *vy, *w, *arr;        /* real-space work arrays [ny][nx] */
    REAL m_old[2], m_new[2], m_appr[2], nonl_v[2];
    F(plan2d) plan;
} F(solver);

static void F(solver_free)(F(solver) * s)
{
    free(s->kx); free(s->ky); free(s->k2); free(s->mask); free(s->lin); free(s->lin2);
    free(s->w_old); free(s->w_new); free(s->w_appr); free(s->nonl);
    free(s->vx_c); free(s->vy_c); free(s->arr_c);
    free(s->vx); free(s->vy); free(s->w); free(s->arr);
    F(plan2d_free)(&s->plan);
}

static int F(solver_init)(F(solver) * s, const orc_params *prm)
{
    memset(s, 0, sizeof(*s));
    int nx = prm->nx, ny = prm->ny, nxh = nx / 2 + 1;
    s->nx = nx; s->ny = ny; s->nxh = nxh; s->size = ny * nxh;
    if (F(plan2d_init)(&s->plan, nx, ny)) return -1;
    size_t H = (size_t)s->size, Nr = (size_t)nx * ny;
    s->kx = (REAL *)malloc(H * sizeof(REAL));
    s->ky = (REAL *)malloc(H * sizeof(REAL));
    s->k2 = (REAL *)malloc(H * sizeof(REAL));
    s->mask = (REAL *)malloc(H * sizeof(REAL));
    s->lin = (REAL *)malloc(H * sizeof(REAL));
    s->lin2 = (REAL *)malloc(H * sizeof(REAL));
    s->w_old = (F(cplx) *)malloc(H * sizeof(F(cplx)));
    s->w_new = (F(cplx) *)malloc(H * sizeof(F(cplx)));
    s->w_appr = (F(cplx) *)malloc(H * sizeof(F(cplx)));
    s->nonl = (F(cplx) *)malloc(H * sizeof(F(cplx)));
    s->vx_c = (F(cplx) *)malloc(H * sizeof(F(cplx)));
    s->vy_c = (F(cplx) *)malloc(H * sizeof(F(cplx)));
    s->arr_c = (F(cplx) *)malloc(H * sizeof(F(cplx)));
    s->vx = (REAL *)malloc(Nr * sizeof(REAL));
    s->vy = (REAL *)malloc(Nr * sizeof(REAL));
    s->w = (REAL *)malloc(Nr * sizeof(REAL));
    s->arr = (REAL *)malloc(Nr * sizeof(REAL));

    /* Normalisation folded into the constants (ActFlow_V3-2.cu:434-436). */
    REAL fnorm = (REAL)(nx * ny);
    s->beta = (REAL)prm->beta / (fnorm * fnorm * fnorm);
    s->lam = (REAL)prm->lam / (fnorm * fnorm);
    s->dt = (REAL)prm->dt;
    REAL dt = s->dt;
    REAL alpha = (REAL)prm->alpha;

    /* Wavenumbers (wavenumber_func, ActFlow_V3-2.cu:1329-1349): 2*pi/L*n in
     * double, stored in REAL; k^2 = ky*ky + kx*kx in REAL. */
    for (int c = 0; c < s->size; c++) {
        int row = c / nxh, col = c % nxh;
        int n = row < ny / 2 + 1 ? row : row - ny;
        s->ky[c] = (REAL)(2.0 * M_PI / (double)(REAL)prm->ly * n);
        s->kx[c] = (REAL)(2.0 * M_PI / (double)(REAL)prm->lx * col);
        s->k2[c] = s->ky[c] * s->ky[c] + s->kx[c] * s->kx[c];
    }
    for (int c = 0; c < s->size; c++) s->mask[c] = (REAL)orc_mask_value(nx, ny, prm->dealias, c % nxh, c / nxh);

    /* Integrating factors (lin_func, ActFlow_V3-2.cu:1020-1033, and the
     * mean-flow scalars, ActFlow_V3-2.cu:704-705).  The general form replaces
     * -(1-k^2)^2 - alpha by -alpha - Gamma0 k^2 - Gamma2 k^4. */
    for (int c = 0; c < s->size; c++) {
        if (prm->if_double) {
            /* the precision form: exp(L dt) and exp(L dt / 2) in double from
             * the double wavenumbers and parameters, rounded to REAL once */
            int row = c / nxh, col = c % nxh;
            int n = row < ny / 2 + 1 ? row : row - ny;
            double kyd = 2.0 * M_PI / prm->ly * n, kxd = 2.0 * M_PI / prm->lx * col;
            double k2d = kyd * kyd + kxd * kxd;
            double Ld = prm->form == 0 ? -(1 - k2d) * (1 - k2d) - prm->alpha
                                       : -prm->alpha - prm->gamma0 * k2d - prm->gamma2 * k2d * k2d;
            s->lin[c] = (REAL)exp(Ld * prm->dt);
            s->lin2[c] = (REAL)exp(Ld * prm->dt / 2);
            continue;
        }
        REAL k2 = s->k2[c];
        REAL L;
        if (prm->form == 0)
            L = -(1 - k2) * (1 - k2) - alpha;
        else
            L = -alpha - (REAL)prm->gamma0 * k2 - (REAL)prm->gamma2 * k2 * k2;
        s->lin[c] = EXPR(L * dt);
        s->lin2[c] = EXPR(L * dt / 2);
    }
    REAL L0 = prm->form == 0 ? -(1 + alpha) : -alpha;
    s->lin_v = EXPR(L0 * dt);
    s->lin2_v = EXPR(L0 * dt / 2);
    return 0;
}

/* The nonlinear term N(w_appr) and the mean-flow right-hand side
 * (nonl_func ActFlow_V3-2.cu:1036-1088 / modified_nonl_func 1090-1161). */
static void F(nonl)(F(solver) * s, double *energy)
{
    int size = s->size, nx = s->nx, ny = s->ny;
    size_t Nr = (size_t)nx * ny;
    /* Biot-Savart (nonl_subfunc_0, ActFlow_V3-2.cu:1176-1180):
     * ux = w * i * ky / k^2, uy = w * i * (-kx) / k^2, for c >= 1. */
#pragma omp parallel for schedule(static)
    for (int c = 1; c < size; c++) {
        F(cplx) w = s->w_appr[c];
        F(cplx) iw = {-w.im, w.re};   /* w * i */
        s->vx_c[c].re = iw.re * s->ky[c] / s->k2[c];
        s->vx_c[c].im = iw.im * s->ky[c] / s->k2[c];
        s->vy_c[c].re = iw.re * -s->kx[c] / s->k2[c];
        s->vy_c[c].im = iw.im * -s->kx[c] / s->k2[c];
    }
    /* The scaled mean velocity goes into the k=0 slot (ActFlow_V3-2.cu:1053-1054). */
    s->vx_c[0].re = s->m_appr[0]; s->vx_c[0].im = 0;
    s->vy_c[0].re = s->m_appr[1]; s->vy_c[0].im = 0;

    /* To real space (ActFlow_V3-2.cu:1057-1059). */
    F(irfft2)(&s->plan, s->vx_c, s->vx);
    F(irfft2)(&s->plan, s->vy_c, s->vy);
    F(irfft2)(&s->plan, s->w_appr, s->w);

    /* Energy of the stage input (ActFlow_V3-2.cu:1118-1127), accumulated in
     * double: E = sum(vx^2 + vy^2) / (2 N^3). */
    if (energy) {
        double acc = 0;
#pragma omp parallel for reduction(+ : acc) schedule(static)
        for (size_t r = 0; r < Nr; r++)
            acc += (double)s->vx[r] * s->vx[r] + (double)s->vy[r] * s->vy[r];
        double n = (double)nx * ny;
        *energy = acc / (2.0 * n * n * n);
    }

    /* Real-space products (nonl_subfunc_1, ActFlow_V3-2.cu:1192-1205):
     * arr = w*vx, w = w*vy, then vx *= |v|^2, vy *= |v|^2. */
#pragma omp parallel for schedule(static)
    for (size_t r = 0; r < Nr; r++) {
        REAL w = s->w[r], vx = s->vx[r], vy = s->vy[r];
        s->arr[r] = w * vx;
        s->w[r] = w * vy;
        REAL v2 = vx * vx + vy * vy;
        s->vx[r] = vx * v2;
        s->vy[r] = vy * v2;
    }
    /* Back to Fourier space (ActFlow_V3-2.cu:1069-1072). */
    F(cplx) *B = s->w_appr, *A = s->arr_c, *C = s->vx_c, *D = s->vy_c;
    F(rfft2)(&s->plan, s->w, B);
    F(rfft2)(&s->plan, s->arr, A);
    F(rfft2)(&s->plan, s->vx, C);
    F(rfft2)(&s->plan, s->vy, D);

    /* Assembly with the mask (nonl_subfunc_2, ActFlow_V3-2.cu:1219-1224):
     * nonl = i * (-kx (lam A + beta D) - ky (lam B - beta C)) * mask. */
    REAL lam = s->lam, beta = s->beta;
#pragma omp parallel for schedule(static)
    for (int c = 0; c < size; c++) {
        REAL tr = -s->kx[c] * (lam * A[c].re + beta * D[c].re) - s->ky[c] * (lam * B[c].re - beta * C[c].re);
        REAL ti = -s->kx[c] * (lam * A[c].im + beta * D[c].im) - s->ky[c] * (lam * B[c].im - beta * C[c].im);
        /* i * (tr + i ti) = -ti + i tr */
        s->nonl[c].re = -ti * s->mask[c];
        s->nonl[c].im = tr * s->mask[c];
    }
    /* Mean-flow right-hand side from the k=0 mode (ActFlow_V3-2.cu:1086-1087). */
    s->nonl_v[0] = -beta * C[0].re;
    s->nonl_v[1] = -beta * D[0].re;
}

/* Hermitian repair of the kx=0 column (reality_func, ActFlow_V3-2.cu:1228-1243). */
static void F(reality)(F(solver) * s)
{
    int nxh = s->nxh, ny = s->ny, size = s->size;
    for (int y = nxh; y < (ny / 2) * nxh; y += nxh) {
        F(cplx) a = s->w_new[y], b = s->w_new[size - y];
        F(cplx) m = {(REAL)0.5f * (a.re + b.re), (REAL)0.5f * (a.im - b.im)};
        s->w_new[y] = m;
        s->w_new[size - y].re = m.re;
        s->w_new[size - y].im = -m.im;
    }
}

/* One time step (ActFlow_V3-2.cu:718-821). */
static void F(step)(F(solver) * s, double *energy)
{
    int size = s->size;
    REAL dt = s->dt;
    /* integrate_func_0 (ActFlow_V3-2.cu:940-955) and the mean copies (729-732). */
    for (int c = 0; c < size; c++) {
        s->w_old[c] = s->w_new[c];
        s->w_appr[c] = s->w_new[c];
        s->w_new[c].re = s->w_new[c].re * s->lin[c];
        s->w_new[c].im = s->w_new[c].im * s->lin[c];
    }
    for (int d = 0; d < 2; d++) { s->m_old[d] = s->m_new[d]; s->m_appr[d] = s->m_new[d]; }

    for (int stage = 1; stage <= 4; stage++) {
        F(nonl)(s, stage == 1 ? energy : NULL);
        F(reality)(s);
        /* integrate_func_1..4 (ActFlow_V3-2.cu:957-1018) and the mean-flow
         * updates (756-759, 778-781, 799-802, 820-821). */
#pragma omp parallel for schedule(static)
        for (int c = 0; c < size; c++) {
            F(cplx) n = s->nonl[c], o = s->w_old[c];
            REAL f;
            switch (stage) {
            case 1:
                f = dt / 6 * s->lin[c];
                s->w_new[c].re += f * n.re; s->w_new[c].im += f * n.im;
                s->w_appr[c].re = s->lin2[c] * (o.re + dt / 2 * n.re);
                s->w_appr[c].im = s->lin2[c] * (o.im + dt / 2 * n.im);
                break;
            case 2:
                f = dt / 3 * s->lin2[c];
                s->w_new[c].re += f * n.re; s->w_new[c].im += f * n.im;
                s->w_appr[c].re = s->lin2[c] * (o.re + dt / 2 * n.re);
                s->w_appr[c].im = s->lin2[c] * (o.im + dt / 2 * n.im);
                break;
            case 3:
                f = dt / 3 * s->lin2[c];
                s->w_new[c].re += f * n.re; s->w_new[c].im += f * n.im;
                s->w_appr[c].re = s->lin[c] * (o.re + dt * n.re);
                s->w_appr[c].im = s->lin[c] * (o.im + dt * n.im);
                break;
            default:
                s->w_new[c].re += dt / 6 * n.re; s->w_new[c].im += dt / 6 * n.im;
                break;
            }
        }
        for (int d = 0; d < 2; d++) {
            REAL nv = s->nonl_v[d];
            switch (stage) {
            case 1:
                s->m_new[d] += dt / 6 * s->lin_v * nv;
                s->m_appr[d] = s->lin2_v * (s->m_old[d] + dt / 2 * nv);
                break;
            case 2:
                s->m_new[d] += dt / 3 * s->lin2_v * nv;
                s->m_appr[d] = s->lin2_v * (s->m_old[d] + dt / 2 * nv);
                break;
            case 3:
                s->m_new[d] += dt / 3 * s->lin2_v * nv;
                s->m_appr[d] = s->lin_v * (s->m_old[d] + dt * nv);
                break;
            default:
                s->m_new[d] += dt / 6 * nv;
                break;
            }
        }
    }
}

int F(orc_run)(const orc_params *prm, REAL *w_hat, REAL *mean, int nsteps, double *energy, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    F(solver) s;
    if (F(solver_init)(&s, prm)) { F(solver_free)(&s); return -1; }
    memcpy(s.w_new, w_hat, sizeof(F(cplx)) * (size_t)s.size);
    s.m_new[0] = mean[0];
    s.m_new[1] = mean[1];
    for (int m = 0; m < nsteps; m++) F(step)(&s, energy ? energy + m : NULL);
    memcpy(w_hat, s.w_new, sizeof(F(cplx)) * (size_t)s.size);
    mean[0] = s.m_new[0];
    mean[1] = s.m_new[1];
    F(solver_free)(&s);
    return 0;
}

int F(orc_rfft2)(int nx, int ny, const REAL *in, REAL *out)
{
    F(plan2d) p;
    if (F(plan2d_init)(&p, nx, ny)) return -1;
    F(rfft2)(&p, in, (F(cplx) *)out);
    F(plan2d_free)(&p);
    return 0;
}

int F(orc_irfft2)(int nx, int ny, const REAL *in, REAL *out)
{
    F(plan2d) p;
    if (F(plan2d_init)(&p, nx, ny)) return -1;
    F(irfft2)(&p, (const F(cplx) *)in, out);
    F(plan2d_free)(&p);
    return 0;
}

#undef F
#undef CAT
#undef CAT_
