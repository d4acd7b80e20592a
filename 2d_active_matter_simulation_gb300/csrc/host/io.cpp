// Snapshot and energy files (reference: save_func ActFlow_V3-2.cu:1245-1266,
// save_energy_func 1268-1278, the continue reader 614-634), plus the host-only
// C entry points that expose them.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <vector>

#include "host.h"

namespace afh {

std::string fmt_g(double v)
{
    char buf[64];
    std::snprintf(buf, sizeof buf, "%g", v);
    return buf;
}

bool write_snapshot(const std::string &path, int nx, int ny, bool fp64, const void *w_hat, const double mean[2])
{
    std::FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    return write_snapshot_to(f, nx, ny, fp64, w_hat, mean);
}

namespace {
const char kRawMagic[8] = {'A', 'F', 'R', 'A', 'W', '1', 0, 0};
}

bool write_snapshot_raw(const std::string &path, int nx, int ny, bool fp64, const void *w_hat, const double mean[2])
{
    std::FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const int hdr[4] = {nx, ny, fp64 ? AM_FP64 : AM_FP32, 0};
    const size_t n = (size_t)ny * (nx / 2 + 1) * 2;
    bool ok = std::fwrite(kRawMagic, 1, 8, f) == 8 && std::fwrite(hdr, sizeof(int), 4, f) == 4 &&
              std::fwrite(w_hat, fp64 ? 8 : 4, n, f) == n && std::fwrite(mean, sizeof(double), 2, f) == 2;
    ok = (std::fclose(f) == 0) && ok;
    return ok;
}

bool read_snapshot_raw(const std::string &path, int nx, int ny, bool fp64, void *w_hat, double mean[2])
{
    std::FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    char magic[8];
    int hdr[4];
    const size_t n = (size_t)ny * (nx / 2 + 1) * 2;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kRawMagic, 8) == 0 &&
              std::fread(hdr, sizeof(int), 4, f) == 4 && hdr[0] == nx && hdr[1] == ny &&
              hdr[2] == (fp64 ? AM_FP64 : AM_FP32) && std::fread(w_hat, fp64 ? 8 : 4, n, f) == n &&
              std::fread(mean, sizeof(double), 2, f) == 2;
    std::fclose(f);
    return ok;
}

bool write_snapshot_to(std::FILE *f, int nx, int ny, bool fp64, const void *w_hat, const double mean[2])
{
    const size_t n = (size_t)ny * (nx / 2 + 1);
    std::vector<char> out;
    out.reserve(n * 26 + 64);
    char buf[64];
    auto put = [&](double v, bool comma) {
        int k = std::snprintf(buf, sizeof buf, comma ? "%g," : "%g", v);
        out.insert(out.end(), buf, buf + k);
    };
    if (fp64) {
        const double *w = (const double *)w_hat;
        for (size_t c = 0; c < 2 * n; c++) put(w[c], true);
        put(mean[0], true);
        put(mean[1], false);
    } else {
        const float *w = (const float *)w_hat;
        for (size_t c = 0; c < 2 * n; c++) put((double)w[c], true);
        put((double)(float)mean[0], true);
        put((double)(float)mean[1], false);
    }
    bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok;
}

bool read_snapshot(const std::string &path, int nx, int ny, bool fp64, void *w_hat, double mean[2])
{
    std::ifstream in(path, std::ios::in | std::ios::binary);
    if (!in.is_open()) return false;
    std::string txt((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    const size_t n = (size_t)ny * (nx / 2 + 1);
    const char *p = txt.c_str();
    const char *end = p + txt.size();
    auto next = [&](double &v) -> bool {
        while (p < end && (*p == ',' || *p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) p++;
        if (p >= end) return false;
        char *q = nullptr;
        errno = 0;
        if (fp64) v = std::strtod(p, &q);
        else v = (double)std::strtof(p, &q);
        if (q == p) return false;
        p = q;
        return true;
    };
    double v;
    for (size_t c = 0; c < 2 * n; c++) {
        if (!next(v)) return false;
        if (fp64) ((double *)w_hat)[c] = v;
        else ((float *)w_hat)[c] = (float)v;
    }
    if (!next(mean[0]) || !next(mean[1])) return false;
    return true;
}

bool append_energy(const std::string &path, long long m0, int count, float dt, const double *energy, bool fp64)
{
    std::FILE *f = std::fopen(path.c_str(), "a");
    if (!f) return false;
    std::string out;
    char buf[96];
    for (int i = 0; i < count; i++) {
        float t = (float)(m0 + i) * dt;
        double e = fp64 ? energy[i] : (double)(float)energy[i];
        int k = std::snprintf(buf, sizeof buf, "%g %g\n", (double)t, e);
        out.append(buf, k);
    }
    bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok;
}

}  // namespace afh

extern "C" {

am_status am_spec_read(const char *dir, am_spec *out, char *err, int errlen)
{
    if (!dir || !out) return AM_ERR_ARG;
    afh::Spec s;
    std::string e;
    int rc = afh::read_spec(dir, s, e);
    if (err && errlen > 0) {
        std::snprintf(err, (size_t)errlen, "%s", e.c_str());
    }
    if (rc) return e.rfind("Error: Unable to open", 0) == 0 ? AM_ERR_IO : AM_ERR_SPEC;
    out->T = s.T;
    out->dt = s.dt;
    out->lx = s.Lx;
    out->ly = s.Ly;
    out->nx = s.Nx;
    out->ny = s.Ny;
    out->lambda = s.lambda;
    out->alpha = s.alpha;
    out->beta = s.beta;
    out->dt_snap = s.dt_snap;
    out->gamma0 = s.gamma0;
    out->gamma2 = s.gamma2;
    out->has_gamma = s.has_gamma ? 1 : 0;
    out->precision = s.precision;
    out->dealias = s.dealias;
    std::snprintf(out->initial, sizeof out->initial, "%s", s.initial.c_str());
    std::snprintf(out->directory, sizeof out->directory, "%s", s.directory.c_str());
    return AM_OK;
}

am_status am_write_snapshot(const char *path, int nx, int ny, int precision, const void *w_hat, const double mean[2])
{
    if (!path || !w_hat || !mean) return AM_ERR_ARG;
    return afh::write_snapshot(path, nx, ny, precision != AM_FP32, w_hat, mean) ? AM_OK : AM_ERR_IO;
}

am_status am_read_snapshot(const char *path, int nx, int ny, int precision, void *w_hat, double mean[2])
{
    if (!path || !w_hat || !mean) return AM_ERR_ARG;
    return afh::read_snapshot(path, nx, ny, precision != AM_FP32, w_hat, mean) ? AM_OK : AM_ERR_IO;
}

am_status am_append_energy(const char *path, long long m0, int count, float dt, const double *energy, int precision)
{
    if (!path || (count > 0 && !energy)) return AM_ERR_ARG;
    return afh::append_energy(path, m0, count, dt, energy, precision != AM_FP32) ? AM_OK : AM_ERR_IO;
}

}  // extern "C"
