// specifications.txt reader (reference: ActFlow_V3-2.cu:320-408).
//
// The file is a sequence of "key:" lines, each followed by one value line.  The
// reference keys and their parsing (stof into float, stoi into int) are kept;
// an unknown key -- including a blank line -- is an error, as in the reference.
// Extension keys accepted in addition (the reference rejects them):
//   precision:  fp32 | fp64 | df64 (double-float)
//   dealias:    reference | half | none
//   Gamma0:, Gamma2:  select the general linear operator -alpha - G0 k^2 - G2 k^4
//   snapshot_binary:  1 = also write ActTurb_snap{i}.raw (exact, used by continue)
#include <fstream>
#include <stdexcept>

#include "host.h"

namespace afh {

namespace {

bool to_float(const std::string &v, float &out)
{
    try {
        out = std::stof(v);
        return true;
    } catch (const std::exception &) {
        return false;
    }
}

bool to_int(const std::string &v, int &out)
{
    try {
        out = std::stoi(v);
        return true;
    } catch (const std::exception &) {
        return false;
    }
}

bool to_double(const std::string &v, double &out)
{
    try {
        out = std::stod(v);
        return true;
    } catch (const std::exception &) {
        return false;
    }
}

}  // namespace

int read_spec(const std::string &dir, Spec &s, std::string &err)
{
    std::ifstream in(dir + "/specifications.txt");
    if (!in.is_open()) {
        err = "Error: Unable to open \"specifications.txt\".";
        return 1;
    }
    std::string line, val;
    while (std::getline(in, line)) {
        bool ok = true;
        auto next = [&]() {
            val.clear();
            std::getline(in, val);
        };
        if (line == "T:") { next(); ok = to_float(val, s.T); }
        else if (line == "dt:") { next(); ok = to_float(val, s.dt); }
        else if (line == "Lx:") { next(); ok = to_float(val, s.Lx); }
        else if (line == "Ly:") { next(); ok = to_float(val, s.Ly); }
        else if (line == "Nx:") { next(); ok = to_int(val, s.Nx); }
        else if (line == "Ny:") { next(); ok = to_int(val, s.Ny); }
        else if (line == "lambda:") { next(); ok = to_float(val, s.lambda); }
        else if (line == "alpha:") { next(); ok = to_float(val, s.alpha); }
        else if (line == "beta:") { next(); ok = to_float(val, s.beta); }
        else if (line == "dt_snap:") { next(); ok = to_float(val, s.dt_snap); }
        else if (line == "initial_condition:") { next(); s.initial = val; }
        else if (line == "save_directory:") { next(); s.directory = val; }
        else if (line == "precision:") {
            next();
            if (val == "fp32") s.precision = AM_FP32;
            else if (val == "fp64") s.precision = AM_FP64;
            else if (val == "df64") s.precision = AM_DF64;
            else ok = false;
        } else if (line == "dealias:") {
            next();
            if (val == "reference") s.dealias = AM_DEALIAS_REFERENCE;
            else if (val == "half") s.dealias = AM_DEALIAS_HALF;
            else if (val == "none") s.dealias = AM_DEALIAS_NONE;
            else ok = false;
        } else if (line == "snapshot_binary:") {
            next();
            int b = 0;
            ok = to_int(val, b);
            s.snapshot_binary = b != 0;
        } else if (line == "Gamma0:") {
            next();
            ok = to_double(val, s.gamma0);
            s.has_gamma = true;
        } else if (line == "Gamma2:") {
            next();
            ok = to_double(val, s.gamma2);
            s.has_gamma = true;
        } else {
            err = "Warning: specification file contains the following unknown specification: " + line +
                  "\nRun the program with the argument \"help\" for the list of specifications.";
            return 1;
        }
        if (!ok) {
            err = "Error: value \"" + val + "\" of specification " + line + " could not be read.";
            return 1;
        }
    }
    return 0;
}

}  // namespace afh
