// Host-side front end of the actflow solver: the reference program's process
// contract (specifications.txt, snapshot and energy files, command line).
#pragma once
#include <cstdio>
#include <string>
#include <vector>

#include "actflow.h"

namespace afh {

// Parsed specifications.txt.  Field defaults are the reference program's
// globals (ActFlow_V3-2.cu:183-204); numeric values are parsed with stof/stoi
// into float/int exactly as the reference does (ActFlow_V3-2.cu:330-391).
struct Spec {
    float T = 100.f;
    float dt = 0.002f;
    float Lx = 250.f;
    float Ly = 250.f;
    int Nx = 1024;
    int Ny = 1024;
    std::string initial = "random";
    std::string directory = "./";
    float dt_snap = 0.5f;
    float lambda = 7.f;
    float alpha = -0.8f;
    float beta = 0.01f;
    // Extension keys (absent from reference files; the reference would reject them).
    bool has_gamma = false;
    double gamma0 = 0.0, gamma2 = 0.0;
    int precision = AM_FP32;
    int dealias = AM_DEALIAS_REFERENCE;
    bool snapshot_binary = false;   // also write the exact binary sidecar ActTurb_snap{i}.raw
};

// Read <dir>/specifications.txt into `s` (which holds the defaults on entry).
// Returns 0, or 1 with a message in `err` (missing file, unknown key --
// ActFlow_V3-2.cu:392-408 -- or a value that does not parse).
int read_spec(const std::string &dir, Spec &s, std::string &err);

// Snapshot text: Ny*(Nx/2+1) pairs "re,im," then "mx,my", every number in the
// default ostream format (six significant digits), ActFlow_V3-2.cu:1261-1263.
// `fp64` selects double values (else float).
bool write_snapshot(const std::string &path, int nx, int ny, bool fp64, const void *w_hat, const double mean[2]);
// Format and write a snapshot into an already opened file, then close it.
bool write_snapshot_to(std::FILE *f, int nx, int ny, bool fp64, const void *w_hat, const double mean[2]);
// Exact binary sidecar: "AFRAW1" magic, nx, ny, precision, the raw half-plane
// values and the mean in double.  Lets `continue` resume bit for bit (the text
// keeps six significant digits, ActFlow_V3-2.cu:1262).
bool write_snapshot_raw(const std::string &path, int nx, int ny, bool fp64, const void *w_hat, const double mean[2]);
// Returns false if absent or not matching (nx, ny, precision).
bool read_snapshot_raw(const std::string &path, int nx, int ny, bool fp64, void *w_hat, double mean[2]);
// Parse a snapshot back (continue path, ActFlow_V3-2.cu:620-631).  Returns
// false if the file cannot be opened or holds fewer numbers than needed.
bool read_snapshot(const std::string &path, int nx, int ny, bool fp64, void *w_hat, double mean[2]);
// Append "t E\n" lines to energy.txt (ActFlow_V3-2.cu:1268-1278); the time
// label is (float)m * dt in float, as the reference computes it.
bool append_energy(const std::string &path, long long m0, int count, float dt, const double *energy, bool fp64);

// The default ostream rendering of a float / double (printf "%g").
std::string fmt_g(double v);

int cli_main(int argc, char **argv);

}  // namespace afh
