// cuFFT floor: the reference program's step with its host synchronisation and
// host energy loop taken out.  A timing comparator, not part of the solver.
//
// The reference (ActFlow_V3-2.cu) advances one IF-RK4 step as 28 cuFFT
// transforms -- per stage 3 C2R and 4 R2C of separate fields on a
// cufftPlan2d plan (ActFlow_V3-2.cu:507-508, 1057-1072, 1111-1145) -- and 21
// grid-stride pointwise kernels (integrate_func_0..4, nonl_subfunc_0..2 and
// reality_func, ActFlow_V3-2.cu:940-1018, 1163-1243), with a
// cudaDeviceSynchronize after every kernel, scalar updates of managed memory
// on the host and, in stage 1, an energy sum over the whole real field on one
// host core (ActFlow_V3-2.cu:1116-1133).  This harness keeps the same
// transforms (same plans, same out-of-place layout), the same pointwise
// kernels with the same data movement, and the mean-flow scalars on the
// device; it drops the syncs, the host loop and the energy entirely, launches
// the pointwise kernels over the whole GPU, and replays one step as a CUDA
// graph.  It is therefore a lower bound on what the reference's own design
// costs per step on this GPU.
//
//   cufft_floor <nx> <ny> <steps> <warmup>
// prints one JSON line {"nx", "ny", "steps", "ms_per_step", "grid_point_steps_per_s"}.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace {

#define CHECK(x)                                                                       \
    do {                                                                               \
        cudaError_t e_ = (x);                                                          \
        if (e_ != cudaSuccess) {                                                       \
            std::fprintf(stderr, "cufft_floor: %s: %s\n", #x, cudaGetErrorString(e_)); \
            std::exit(2);                                                              \
        }                                                                              \
    } while (0)
#define CHECK_FFT(x)                                                           \
    do {                                                                       \
        cufftResult r_ = (x);                                                  \
        if (r_ != CUFFT_SUCCESS) {                                             \
            std::fprintf(stderr, "cufft_floor: %s: cufft error %d\n", #x, (int)r_); \
            std::exit(2);                                                      \
        }                                                                      \
    } while (0)

struct Mean {             // scaled mean velocity and its right-hand side
    float old_[2], new_[2], appr[2], rhs[2];
};

struct Fields {
    int size;                              // Ny * (Nx/2 + 1)
    int nxh, ny;
    float dt, lam, beta, lin_v, lin2_v;    // lam, beta divided by N^2, N^3
    cufftComplex *w_old, *w_new, *w_appr, *vx, *vy, *arr, *nonl;
    float *rw, *rarr, *rvx, *rvy;          // real-space fields
    const float *kx, *ky, *k2, *mask, *lin, *lin2;
    Mean *mean;
};

__device__ inline cufftComplex cadd(cufftComplex a, cufftComplex b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ inline cufftComplex cscale(cufftComplex a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ inline int gtid() { return blockIdx.x * blockDim.x + threadIdx.x; }
__device__ inline int gstride() { return blockDim.x * gridDim.x; }

// stage start: w_old = w_appr = w_new, w_new *= lin; the mean likewise
__global__ void k_start(Fields f)
{
    for (int c = gtid(); c < f.size; c += gstride()) {
        const cufftComplex w = f.w_new[c];
        f.w_old[c] = w;
        f.w_appr[c] = w;
        f.w_new[c] = cscale(w, f.lin[c]);
    }
    if (gtid() == 0)
        for (int d = 0; d < 2; d++) f.mean->old_[d] = f.mean->appr[d] = f.mean->new_[d];
}

// velocity from vorticity (stream function), mean velocity in the k = 0 slot
__global__ void k_velocity(Fields f)
{
    for (int c = gtid(); c < f.size; c += gstride()) {
        if (c == 0) {
            f.vx[0] = make_float2(f.mean->appr[0], 0.f);
            f.vy[0] = make_float2(f.mean->appr[1], 0.f);
            continue;
        }
        const cufftComplex w = f.w_appr[c];
        const float qx = f.ky[c] / f.k2[c], qy = -f.kx[c] / f.k2[c];
        f.vx[c] = make_float2(-w.y * qx, w.x * qx);
        f.vy[c] = make_float2(-w.y * qy, w.x * qy);
    }
}

// the four real-space products, in the reference's two sweeps
__global__ void k_products(Fields f, int n)
{
    for (int r = gtid(); r < n; r += gstride()) {
        const float w = f.rw[r];
        f.rarr[r] = w * f.rvx[r];
        f.rw[r] = w * f.rvy[r];
    }
    for (int r = gtid(); r < n; r += gstride()) {
        const float vx = f.rvx[r], vy = f.rvy[r], s = vx * vx + vy * vy;
        f.rvx[r] = vx * s;
        f.rvy[r] = vy * s;
    }
}

// nonlinear term from the transformed products, masked; mean-flow RHS
__global__ void k_assemble(Fields f)
{
    for (int c = gtid(); c < f.size; c += gstride()) {
        const cufftComplex A = f.arr[c], B = f.w_appr[c], C = f.vx[c], D = f.vy[c];
        const float re = -f.kx[c] * (f.lam * A.x + f.beta * D.x) - f.ky[c] * (f.lam * B.x - f.beta * C.x);
        const float im = -f.kx[c] * (f.lam * A.y + f.beta * D.y) - f.ky[c] * (f.lam * B.y - f.beta * C.y);
        f.nonl[c] = make_float2(-im * f.mask[c], re * f.mask[c]);
    }
    if (gtid() == 0) {
        f.mean->rhs[0] = -f.beta * f.vx[0].x;
        f.mean->rhs[1] = -f.beta * f.vy[0].x;
    }
}

// Hermitian symmetry of the kx = 0 column of w_new
__global__ void k_reality(Fields f)
{
    for (int y = gtid() + 1; y < f.ny / 2; y += gstride()) {
        const int a = y * f.nxh, b = f.size - a;
        const cufftComplex u = f.w_new[a], v = f.w_new[b];
        const cufftComplex m = make_float2(0.5f * (u.x + v.x), 0.5f * (u.y - v.y));
        f.w_new[a] = m;
        f.w_new[b] = make_float2(m.x, -m.y);
    }
}

// stage combination s = 1..4 (the reference's stage inputs), mean alike
template <int S>
__global__ void k_combine(Fields f)
{
    const float dt = f.dt;
    for (int c = gtid(); c < f.size; c += gstride()) {
        const cufftComplex n = f.nonl[c], o = f.w_old[c];
        if (S == 1) {
            f.w_new[c] = cadd(f.w_new[c], cscale(n, dt / 6 * f.lin[c]));
            f.w_appr[c] = cscale(cadd(o, cscale(n, dt / 2)), f.lin2[c]);
        } else if (S == 2) {
            f.w_new[c] = cadd(f.w_new[c], cscale(n, dt / 3 * f.lin2[c]));
            f.w_appr[c] = cscale(cadd(o, cscale(n, dt / 2)), f.lin2[c]);
        } else if (S == 3) {
            f.w_new[c] = cadd(f.w_new[c], cscale(n, dt / 3 * f.lin2[c]));
            f.w_appr[c] = cscale(cadd(o, cscale(n, dt)), f.lin[c]);
        } else {
            f.w_new[c] = cadd(f.w_new[c], cscale(n, dt / 6));
        }
    }
    if (gtid() == 0) {
        Mean &m = *f.mean;
        for (int d = 0; d < 2; d++) {
            const float r = m.rhs[d];
            if (S == 1) {
                m.new_[d] += dt / 6 * f.lin_v * r;
                m.appr[d] = f.lin2_v * (m.old_[d] + dt / 2 * r);
            } else if (S == 2) {
                m.new_[d] += dt / 3 * f.lin2_v * r;
                m.appr[d] = f.lin2_v * (m.old_[d] + dt / 2 * r);
            } else if (S == 3) {
                m.new_[d] += dt / 3 * f.lin2_v * r;
                m.appr[d] = f.lin_v * (m.old_[d] + dt * r);
            } else {
                m.new_[d] += dt / 6 * r;
            }
        }
    }
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 5) {
        std::fprintf(stderr, "usage: cufft_floor <nx> <ny> <steps> <warmup>\n");
        return 1;
    }
    const int nx = std::atoi(argv[1]), ny = std::atoi(argv[2]), steps = std::atoi(argv[3]),
              warmup = std::atoi(argv[4]);
    if (nx < 8 || ny < 8 || steps < 1 || warmup < 0) return 1;
    const int nxh = nx / 2 + 1, size = ny * nxh;
    // the benchmark workload's parameters in the reference's normalised units
    const double ell = std::sqrt(-2.0 * 2.5e-5 / -0.045), tau = std::pow(ell, 4) / 2.5e-5;
    const float alpha = (float)(tau * -0.8 - 1.0), beta = (float)(0.01 * ell * ell / tau), lam = 3.5f;
    const float L = (float)(2.0 * M_PI / ell), dt = (float)(1e-4 / tau);

    std::vector<float> kx(size), ky(size), k2(size), mask(size), lin(size), lin2(size);
    for (int c = 0; c < size; c++) {
        const int row = c / nxh, col = c % nxh, n = row < ny / 2 + 1 ? row : row - ny;
        ky[c] = (float)(2.0 * M_PI / L * n);
        kx[c] = (float)(2.0 * M_PI / L * col);
        k2[c] = kx[c] * kx[c] + ky[c] * ky[c];
        // 1/2 rule; the mask's values do not change the work
        mask[c] = 16.0 * ((double)col * col / ((double)nx * nx) + (double)n * n / ((double)ny * ny)) <= 1.0 ? 1.f : 0.f;
        const float Lk = -(1 - k2[c]) * (1 - k2[c]) - alpha;
        lin[c] = std::exp(Lk * dt);
        lin2[c] = std::exp(Lk * dt / 2);
    }
    // a seeded band-limited field: modes 1 <= |k| <= 8 (in units of the box)
    std::vector<cufftComplex> w0(size, make_float2(0.f, 0.f));
    unsigned long long s = 7;
    auto uni = [&s]() {
        s = s * 6364136223846793005ULL + 1442695040888963407ULL;
        return (double)(s >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int row = 0; row < ny; row++)
        for (int col = 0; col < nxh; col++) {
            const int n = row < ny / 2 + 1 ? row : row - ny;
            const int r2 = n * n + col * col;
            if (r2 >= 1 && r2 <= 64 && !(col == 0 && n <= 0))
                w0[row * nxh + col] = make_float2((float)(uni() - 0.5) * 1e3f, (float)(uni() - 0.5) * 1e3f);
        }

    Fields f{};
    f.size = size;
    f.nxh = nxh;
    f.ny = ny;
    const float fn = (float)nx * ny;
    f.dt = dt;
    f.lam = lam / (fn * fn);
    f.beta = beta / (fn * fn * fn);
    f.lin_v = std::exp(-(1 + alpha) * dt);
    f.lin2_v = std::exp(-(1 + alpha) * dt / 2);
    cufftComplex **cf[] = {&f.w_old, &f.w_new, &f.w_appr, &f.vx, &f.vy, &f.arr, &f.nonl};
    for (auto p : cf) CHECK(cudaMalloc(p, (size_t)size * sizeof(cufftComplex)));
    float **rf[] = {&f.rw, &f.rarr, &f.rvx, &f.rvy};
    for (auto p : rf) CHECK(cudaMalloc(p, (size_t)2 * size * sizeof(float)));
    const std::vector<float> *tabs[] = {&kx, &ky, &k2, &mask, &lin, &lin2};
    const float **tp[] = {&f.kx, &f.ky, &f.k2, &f.mask, &f.lin, &f.lin2};
    for (int i = 0; i < 6; i++) {
        float *d = nullptr;
        CHECK(cudaMalloc(&d, (size_t)size * sizeof(float)));
        CHECK(cudaMemcpy(d, tabs[i]->data(), (size_t)size * sizeof(float), cudaMemcpyHostToDevice));
        *tp[i] = d;
    }
    CHECK(cudaMalloc(&f.mean, sizeof(Mean)));
    CHECK(cudaMemset(f.mean, 0, sizeof(Mean)));
    CHECK(cudaMemcpy(f.w_new, w0.data(), (size_t)size * sizeof(cufftComplex), cudaMemcpyHostToDevice));

    cudaStream_t st;
    CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cufftHandle fwd, inv;
    CHECK_FFT(cufftPlan2d(&fwd, ny, nx, CUFFT_R2C));
    CHECK_FFT(cufftPlan2d(&inv, ny, nx, CUFFT_C2R));
    CHECK_FFT(cufftSetStream(fwd, st));
    CHECK_FFT(cufftSetStream(inv, st));
    int dev = 0, sms = 0;
    CHECK(cudaGetDevice(&dev));
    CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = sms * 8, block = 256;
    const int nreal = nx * ny;

    auto stage = [&](int s) {
        k_velocity<<<grid, block, 0, st>>>(f);
        CHECK_FFT(cufftExecC2R(inv, f.vx, f.rvx));
        CHECK_FFT(cufftExecC2R(inv, f.vy, f.rvy));
        CHECK_FFT(cufftExecC2R(inv, f.w_appr, f.rw));
        k_products<<<grid, block, 0, st>>>(f, nreal);
        CHECK_FFT(cufftExecR2C(fwd, f.rw, f.w_appr));
        CHECK_FFT(cufftExecR2C(fwd, f.rarr, f.arr));
        CHECK_FFT(cufftExecR2C(fwd, f.rvx, f.vx));
        CHECK_FFT(cufftExecR2C(fwd, f.rvy, f.vy));
        k_assemble<<<grid, block, 0, st>>>(f);
        k_reality<<<grid, block, 0, st>>>(f);
        if (s == 1) k_combine<1><<<grid, block, 0, st>>>(f);
        if (s == 2) k_combine<2><<<grid, block, 0, st>>>(f);
        if (s == 3) k_combine<3><<<grid, block, 0, st>>>(f);
        if (s == 4) k_combine<4><<<grid, block, 0, st>>>(f);
    };
    cudaGraph_t g;
    cudaGraphExec_t ge;
    CHECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    k_start<<<grid, block, 0, st>>>(f);
    for (int s = 1; s <= 4; s++) stage(s);
    CHECK(cudaStreamEndCapture(st, &g));
    CHECK(cudaGraphInstantiate(&ge, g, 0));

    for (int i = 0; i < warmup; i++) CHECK(cudaGraphLaunch(ge, st));
    CHECK(cudaStreamSynchronize(st));
    cudaEvent_t e0, e1;
    CHECK(cudaEventCreate(&e0));
    CHECK(cudaEventCreate(&e1));
    CHECK(cudaEventRecord(e0, st));
    for (int i = 0; i < steps; i++) CHECK(cudaGraphLaunch(ge, st));
    CHECK(cudaEventRecord(e1, st));
    CHECK(cudaEventSynchronize(e1));
    float ms = 0;
    CHECK(cudaEventElapsedTime(&ms, e0, e1));
    cufftComplex w00;
    CHECK(cudaMemcpy(&w00, f.w_new + 1, sizeof(w00), cudaMemcpyDeviceToHost));
    const double per = ms / steps;
    std::printf("{\"nx\": %d, \"ny\": %d, \"steps\": %d, \"warmup\": %d, \"ms_per_step\": %.6f, "
                "\"grid_point_steps_per_s\": %.6e, \"finite\": %s}\n",
                nx, ny, steps, warmup, per, (double)nx * ny / (per * 1e-3),
                std::isfinite(w00.x) && std::isfinite(w00.y) ? "true" : "false");
    cufftDestroy(fwd);
    cufftDestroy(inv);
    return 0;
}
