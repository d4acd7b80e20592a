// The drop-in program (reference: main, ActFlow_V3-2.cu:214-878).
//
//   actflow <dir>    run the simulation described by <dir>/specifications.txt
//   actflow help|h   usage
//   actflow spec     write specifications.txt with the default settings
//   actflow math     write theory.tex with the model equations
//
// Process contract kept from the reference: exit 0 on success, 1 on a bad
// argument count, a spec error, an unknown initial condition, a missing
// continue snapshot, an unwritable output file or a NaN in w(0,0); the same
// output files and formats; the same step numbering (m starts at 1 for a fresh
// run and at cont_snap*snap for a continued one; energy line m carries m*dt and
// the energy of the state entering step m; snapshot m/snap is written after
// every step m with m % snap == 0).  Differences: CUDA errors end the program
// with exit 1 and a message instead of std::terminate (cudaErr.h:41-59), a
// value that does not parse is reported instead of throwing, and dt_snap < dt/2
// (snap = 0, undefined behaviour in the reference, ActFlow_V3-2.cu:421, 824) is
// rejected.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <random>
#include <thread>
#include <vector>

#include "host.h"

namespace afh {

namespace {

const char *HELP =
    "\n--------------------------------------------------\n"
    "actflow: GB300 solver for the 2-D continuum model of active turbulence\n"
    "(vorticity form of the Wensink / James-Bos-Wilczek model, integrating-factor RK4).\n\n"
    "usage:\n"
    "  actflow <dir>    run the simulation configured in <dir>/specifications.txt;\n"
    "                   snapshots ActTurb_snap{i}.bin and energy.txt go to save_directory\n"
    "  actflow help     print this text\n"
    "  actflow spec     write specifications.txt with the default settings\n"
    "  actflow math     write theory.tex with the model equations\n\n"
    "specifications.txt holds \"key:\" lines, each followed by its value:\n"
    "  T, dt, Lx, Ly, Nx, Ny, lambda, alpha, beta, dt_snap,\n"
    "  initial_condition (random [n] | blank | continue [T_ext [snapshot]] |\n"
    "                     bandlimited <seed> [kmin kmax rms]),\n"
    "  save_directory,\n"
    "  optional: precision (fp32|fp64|df64), dealias (reference|half|none), Gamma0, Gamma2,\n"
    "            snapshot_binary (1: exact ActTurb_snap{i}.raw beside each snapshot)\n"
    "--------------------------------------------------\n";

int write_default_spec()
{
    Spec s;
    std::ofstream f("specifications.txt", std::ios::out);
    if (!f.is_open()) {
        std::cerr << "Error: unable to create example file" << std::endl;
        return 1;
    }
    f << "T:\n" << fmt_g(s.T) << "\ndt:\n" << fmt_g(s.dt) << "\nLx:\n" << fmt_g(s.Lx) << "\nLy:\n"
      << fmt_g(s.Ly) << "\nNx:\n" << s.Nx << "\nNy:\n" << s.Ny << "\nlambda:\n" << fmt_g(s.lambda)
      << "\nalpha:\n" << fmt_g(s.alpha) << "\nbeta:\n" << fmt_g(s.beta) << "\ndt_snap:\n" << fmt_g(s.dt_snap)
      << "\ninitial_condition:\n" << s.initial << "\nsave_directory:\n" << s.directory;
    f.close();
    std::cout << "example has been created" << std::endl;
    return 0;
}

int write_theory()
{
    std::ofstream f("theory.tex", std::ios::out);
    if (!f.is_open()) {
        std::cerr << "Error: unable to create theory file" << std::endl;
        return 1;
    }
    f << "\\documentclass{article}\n\\usepackage{amsmath}\n\\begin{document}\n"
         "\\section*{Model}\n"
         "The vorticity $\\omega = \\partial_x u_y - \\partial_y u_x$ of an incompressible 2-D active "
         "fluid (Wensink et al.; normalised form of James, Bos and Wilczek) obeys\n"
         "\\begin{equation}\n"
         "\\partial_t \\omega + \\lambda\\, (\\mathbf u\\cdot\\nabla)\\omega = "
         "-(1+\\nabla^2)^2\\omega - \\alpha\\,\\omega - \\beta\\, \\nabla\\times(|\\mathbf u|^2 \\mathbf u)\n"
         "\\end{equation}\n"
         "on a doubly periodic box.  The mean velocity, which the vorticity does not determine, follows\n"
         "\\begin{equation}\n"
         "\\partial_t \\langle\\mathbf u\\rangle = -(1+\\alpha)\\langle\\mathbf u\\rangle "
         "- \\beta\\,\\langle|\\mathbf u|^2 \\mathbf u\\rangle .\n"
         "\\end{equation}\n"
         "In Fourier space $\\hat u_x = i k_y \\hat\\omega / k^2$, $\\hat u_y = -i k_x \\hat\\omega / k^2$; "
         "the linear part $L(k) = -(1-k^2)^2 - \\alpha$ is integrated exactly by the factor "
         "$e^{L(k)\\,\\Delta t}$ and the nonlinear part by a fourth-order Runge--Kutta scheme.\n"
         "With the optional keys Gamma0, Gamma2 the linear part is "
         "$L(k) = -\\alpha - \\Gamma_0 k^2 - \\Gamma_2 k^4$ and the mean decays with $-\\alpha$.\n"
         "\\end{document}"
      << std::endl;
    f.close();
    std::cout << "a Latex file \"theory.tex\" has been created" << std::endl;
    return 0;
}

bool exists(const std::string &path)
{
    std::ifstream f(path);
    return f.good();
}

std::string snap_path(const std::string &dir, long long i) { return dir + "/ActTurb_snap" + std::to_string(i) + ".bin"; }
std::string raw_path(const std::string &dir, long long i) { return dir + "/ActTurb_snap" + std::to_string(i) + ".raw"; }

// Snapshots without stalling the step loop.  The file is opened on the calling
// thread (so an unwritable directory fails at the same step as in the
// reference, ActFlow_V3-2.cu:824-839), the state is copied to one of two host
// buffers, and a background thread formats and writes the text (the slow part
// at large grids) while the GPU runs the next steps.  A second snapshot waits
// for the first writer to finish before reusing its buffer.
class SnapshotWriter {
  public:
    SnapshotWriter(int nx, int ny, bool fp64, bool raw, size_t bytes) : nx_(nx), ny_(ny), fp64_(fp64), raw_(raw)
    {
        buf_[0].resize(bytes);
        buf_[1].resize(bytes);
    }
    ~SnapshotWriter() { finish(); }
    // Buffer the next snapshot's state goes into.
    void *buffer() { return buf_[cur_].data(); }
    double *mean() { return mean_[cur_]; }
    // Hand the current buffer to the writer thread.  False if the file cannot
    // be created or an earlier write failed.
    bool submit(const std::string &dir, long long index)
    {
        std::FILE *f = std::fopen(snap_path(dir, index).c_str(), "wb");
        if (!f) return false;
        if (!finish()) {
            std::fclose(f);
            return false;
        }
        const int b = cur_;
        const std::string rp = raw_ ? raw_path(dir, index) : std::string();
        th_ = std::thread([this, f, b, rp]() {
            bool ok = write_snapshot_to(f, nx_, ny_, fp64_, buf_[b].data(), mean_[b]);
            if (!rp.empty()) ok = write_snapshot_raw(rp, nx_, ny_, fp64_, buf_[b].data(), mean_[b]) && ok;
            ok_ = ok;
        });
        cur_ ^= 1;
        return true;
    }
    // Wait for the writer; false if its write failed.
    bool finish()
    {
        if (th_.joinable()) th_.join();
        return ok_;
    }

  private:
    int nx_, ny_;
    bool fp64_, raw_;
    std::vector<unsigned char> buf_[2];
    double mean_[2][2] = {{0, 0}, {0, 0}};
    int cur_ = 0;
    std::thread th_;
    bool ok_ = true;
};

}  // namespace

int cli_main(int argc, char **argv)
{
    if (argc != 2) {
        std::cerr << "Exactly one argument is expected: the simulation directory, or help / spec / math."
                  << std::endl;
        return 1;
    }
    if (!std::strcmp(argv[1], "help") || !std::strcmp(argv[1], "h")) {
        std::cout << HELP << std::endl;
        return 0;
    }
    if (!std::strcmp(argv[1], "spec")) return write_default_spec();
    if (!std::strcmp(argv[1], "math")) return write_theory();

    Spec s;
    s.directory = argv[1];
    std::cout << "reading the specifications (path=" << s.directory << "/specifications.txt)" << std::endl;
    std::string err;
    if (read_spec(s.directory, s, err)) {
        std::cerr << err << std::endl;
        return 1;
    }
    const std::string &dir = s.directory;
    // Derived quantities (ActFlow_V3-2.cu:409-421), in float like the reference.
    long long M = (long long)std::round(s.T / s.dt);
    const int Nxh = s.Nx / 2 + 1;
    const size_t size = (size_t)s.Ny * Nxh;
    const long long snap = (long long)std::round(s.dt_snap / s.dt);
    if (snap <= 0) {
        std::cerr << "Error: dt_snap must be at least dt/2 (snapshot interval of 0 steps)." << std::endl;
        return 1;
    }
    const bool fp64 = s.precision != AM_FP32;   // host values in double (FP64, double-float)
    std::cout << "--------------------------------------------------\n"
              << "T = " << fmt_g(s.T) << "\ndt = " << fmt_g(s.dt) << "\nM = " << M << "\nLx = " << fmt_g(s.Lx)
              << "\nLy = " << fmt_g(s.Ly) << "\nNx = " << s.Nx << "\nNy = " << s.Ny
              << "\nalpha = " << fmt_g(s.alpha) << "\nbeta = " << fmt_g(s.beta) << "\nlambda = " << fmt_g(s.lambda)
              << "\ninitial condition: " << s.initial << "\ntotal amount of snapshots: " << M / snap
              << "\nprecision: " << (s.precision == AM_DF64 ? "df64" : fp64 ? "fp64" : "fp32")
              << "\n--------------------------------------------------" << std::endl;

    am_params p{};
    p.nx = s.Nx;
    p.ny = s.Ny;
    p.lx = s.Lx;
    p.ly = s.Ly;
    p.dt = s.dt;
    p.lambda = s.lambda;
    p.alpha = s.alpha;
    p.beta = s.beta;
    p.gamma0 = s.gamma0;
    p.gamma2 = s.gamma2;
    p.form = s.has_gamma ? AM_FORM_GENERAL : AM_FORM_REFERENCE;
    p.dealias = s.dealias;
    p.precision = s.precision;
    am_handle *h = nullptr;
    am_status st = am_create(&p, &h);
    if (st) {
        std::cerr << "Error: unable to set up the solver: " << am_status_string(st) << std::endl;
        return 1;
    }
    struct Guard {
        am_handle *h;
        ~Guard() { am_destroy(h); }
    } guard{h};

    const size_t elem = fp64 ? sizeof(double) : sizeof(float);
    std::vector<unsigned char> w(size * 2 * elem);
    double mean[2] = {0.0, 0.0};
    long long m = 1;   // step counter (ActFlow_V3-2.cu:529)

    const std::string &ic = s.initial;
    if (ic.substr(0, 6) == "random") {
        // Uniform(-1, 1) real-space field from a clock-seeded mt19937_64
        // (ActFlow_V3-2.cu:535-559), then R2C, mask and w(0,0) = 0.
        std::cout << "generating random initial condition" << std::endl;
        int seed = (int)std::chrono::system_clock::to_time_t(std::chrono::system_clock::now());
        if (ic.find(' ') != std::string::npos) {
            int d = 0;
            try {
                d = std::stoi(ic.substr(ic.find(' ') + 1));
            } catch (const std::exception &) {
                d = 0;
            }
            if (d == 0) {
                std::cerr << "Error: unknown specification for the initial condition" << std::endl;
                return 1;
            }
            seed /= d;
        }
        std::mt19937_64 gen(seed);
        std::uniform_real_distribution<float> dist(-1.f, 1.f);
        std::vector<unsigned char> real((size_t)s.Nx * s.Ny * elem);
        for (size_t r = 0; r < 2 * size; r++) {
            int col = (int)(r % (size_t)(s.Nx + 2));
            if (col >= s.Nx) continue;   // padding columns of the in-place layout
            float v = dist(gen);
            size_t k = (r / (size_t)(s.Nx + 2)) * s.Nx + col;
            if (fp64) ((double *)real.data())[k] = v;
            else ((float *)real.data())[k] = v;
        }
        st = am_set_state_real(h, real.data(), mean, 1);
    } else if (ic == "blank") {
        std::cout << "generating blank initial condition" << std::endl;
        std::vector<unsigned char> real((size_t)s.Nx * s.Ny * elem, 0);
        st = am_set_state_real(h, real.data(), mean, 1);
    } else if (ic.substr(0, 11) == "bandlimited") {
        // Extension: seeded band-limited field, "bandlimited <seed> [kmin kmax rms]".
        unsigned long long seed = 0;
        double kmin = 1, kmax = 8, rms = 0.01;
        int n = std::sscanf(ic.c_str() + 11, "%llu %lf %lf %lf", &seed, &kmin, &kmax, &rms);
        if (n != 1 && n != 4) {
            std::cerr << "Error: unknown specification for the initial condition" << std::endl;
            return 1;
        }
        std::vector<double> wd(size * 2);
        if (am_ic_bandlimited(s.Nx, s.Ny, seed, kmin, kmax, rms, wd.data())) {
            std::cerr << "Error: band-limited initial condition does not fit the grid" << std::endl;
            return 1;
        }
        if (fp64) std::memcpy(w.data(), wd.data(), wd.size() * sizeof(double));
        else
            for (size_t i = 0; i < wd.size(); i++) ((float *)w.data())[i] = (float)wd[i];
        st = am_set_state(h, w.data(), mean);
    } else if (ic.substr(0, 8) == "continue") {
        // Resume from the last contiguous snapshot (ActFlow_V3-2.cu:567-647).
        long long cont = -1;
        for (long long i = 0; i < 1000000; i++) {
            if (exists(snap_path(dir, i))) cont = i;
            else break;
        }
        if (cont == -1) {
            std::cerr << "Error: Tried to continue from previous simulation, but no previous snapshot was found."
                      << std::endl;
            return 1;
        }
        if (ic.find(' ') != std::string::npos) {
            std::string args = ic.substr(ic.find(' ') + 1);
            try {
                if (args.find(' ') != std::string::npos) {
                    cont = std::stoi(args.substr(args.find(' ') + 1));
                    M = (long long)(float)(cont * snap + std::round(std::stof(args.substr(0, args.find(' '))) / s.dt));
                } else {
                    M = (long long)(float)(cont * snap + std::round(std::stof(args) / s.dt));
                }
            } catch (const std::exception &) {
                std::cerr << "Error: unknown specification for the initial condition" << std::endl;
                return 1;
            }
        }
        std::cout << "continue execution from snapshot " << cont << std::endl;
        m = cont * snap;
        // An exact binary sidecar of the same snapshot, when present, is used
        // instead of the six-digit text.
        if (read_snapshot_raw(raw_path(dir, cont), s.Nx, s.Ny, fp64, w.data(), mean)) {
            std::cout << "using the exact binary copy " << raw_path(dir, cont) << std::endl;
        } else if (!read_snapshot(snap_path(dir, cont), s.Nx, s.Ny, fp64, w.data(), mean)) {
            std::cerr << "Error: unable to open previous simulation" << std::endl;
            return 1;
        }
        st = am_set_state(h, w.data(), mean);
    } else {
        std::cerr << "Error: unknown specification for the initial condition" << std::endl;
        return 1;
    }
    if (st) {
        std::cerr << "Error: " << am_status_string(st) << ": " << am_last_error(h) << std::endl;
        return 1;
    }
    SnapshotWriter writer(s.Nx, s.Ny, fp64, s.snapshot_binary, w.size());
    if (m == 1) {
        // A fresh start saves the processed initial condition as snapshot 0
        // (ActFlow_V3-2.cu:660-694).
        std::cout << "processing the initial condition" << std::endl;
        if ((st = am_get_state(h, writer.buffer(), writer.mean())) || !writer.submit(dir, 0)) {
            std::cerr << "Error: unable to create snapshot file" << std::endl;
            return 1;
        }
    }

    std::cout << "initializing the time stepping" << std::endl;
    auto t0 = std::chrono::high_resolution_clock::now();
    const std::string efile = dir + "/energy.txt";
    std::vector<double> energy;
    while (m <= M) {
        // Run up to and including the next snapshot step.
        long long next = ((m + snap - 1) / snap) * snap;
        if (m % snap == 0) next = m;
        long long last = next < M ? next : M;
        int k = (int)(last - m + 1);
        energy.assign(k, 0.0);
        int nan_at = -1;
        st = am_step(h, k, energy.data(), &nan_at);
        if (st && st != AM_ERR_NAN) {
            std::cerr << "Error: " << am_status_string(st) << ": " << am_last_error(h) << std::endl;
            return 1;
        }
        int good = st == AM_ERR_NAN ? nan_at + 1 : k;
        if (!append_energy(efile, m, good, s.dt, energy.data(), fp64)) {
            std::cerr << "Error: failed to save the mean energy" << std::endl;
            return 1;
        }
        long long m_end = m + good - 1;
        bool at_snap = m_end % snap == 0 && (st != AM_ERR_NAN || good == k);
        if (at_snap) {
            const void *sw = writer.buffer();
            if (am_get_state(h, writer.buffer(), writer.mean()) || !writer.submit(dir, m_end / snap)) {
                std::cerr << "Error: unable to create snapshot file" << std::endl;
                return 1;
            }
            std::chrono::duration<double> el = std::chrono::high_resolution_clock::now() - t0;
            double w0r = fp64 ? ((const double *)sw)[0] : ((const float *)sw)[0];
            double w0i = fp64 ? ((const double *)sw)[1] : ((const float *)sw)[1];
            std::cout << "\r" << m_end << " / " << M << " timesteps done in " << el.count() << "s, w[0]=("
                      << fmt_g(w0r) << "," << fmt_g(w0i) << ")    " << std::flush;
        }
        if (st == AM_ERR_NAN) {
            writer.finish();
            std::cerr << "\nError: array contains nan values after " << m_end << " timesteps" << std::endl;
            return 1;
        }
        m = last + 1;
    }
    if (!writer.finish()) {
        std::cerr << "Error: unable to create snapshot file" << std::endl;
        return 1;
    }
    std::chrono::duration<double> el = std::chrono::high_resolution_clock::now() - t0;
    std::cout << "\nprogram finished successfully after " << el.count() << "s.\n" << std::endl;
    return 0;
}

}  // namespace afh

extern "C" int am_cli_main(int argc, char **argv) { return afh::cli_main(argc, argv); }
