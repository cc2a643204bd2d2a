// host_io.cpp -- the reference's ASCII inputs, read the way its drivers read them.
//
// The drivers (src/calculateNNMap.cu:42-129, src/calculateNNMap_twoPop.cu:79-121,
// src/calculateNMapMap.cu) load every table through g3lhalo::Function /
// g3lhalo::Function2D, the HOD vectors through g3lhalo::Params, the cosmology through
// g3lhalo::Cosmology and the aperture triplets with a bare stream loop.  These entry
// points give a C-ABI caller the same arrays from the same files:
//   - whitespace-separated numbers parsed by C++ stream extraction, reading stopping
//     at the first token that is not a number (as `while (input >> x >> y)` does);
//   - 1-D tables: linear interpolation on the file's points, the default value outside
//     [x_first, x_last) (src/Function.cpp:52-73), sampled at min + i (max-min)/N or
//     exp(log min + i log(max/min)/N) (src/Function.cpp:89-124);
//   - 2-D tables: the nearest-bin lookup of src/Function2D.cpp:46-95 over the file's
//     values in file order, the first coordinate linear and the second logarithmic.
// Where the reference exits, or continues with undefined values (an unreadable
// file, an unknown or missing parameter, too few 2-D rows), these return
// G3L_ERR_INVALID and set g3l_last_error().
#include <cmath>
#include <fstream>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "g3l_gpu.h"
#include "host_internal.h"

namespace {

int fail(const std::string &msg)
{
    g3l::host::set_error(msg);
    return G3L_ERR_INVALID;
}

int fail_nomem(const char *what)
{
    g3l::host::set_error(std::string(what) + ": host allocation failed");
    return G3L_ERR_NOMEM;
}

// value at x of the piecewise-linear 1-D table (src/Function.cpp:52-73)
double at_1d(const std::vector<double> &xs, const std::vector<double> &ys, double x, double def)
{
    if (x > xs.back() || x < xs.front()) return def;
    for (size_t i = 0; i + 1 < xs.size(); ++i)
        if (xs[i] <= x && xs[i + 1] > x) {
            const double a = (ys[i + 1] - ys[i]) / (xs[i + 1] - xs[i]);
            return a * (x - xs[i]) + ys[i];
        }
    return def;
}

// "name value" lines, '#' comments and empty lines skipped (src/Params.cpp:20-36,
// src/Cosmology.cpp:18-34).  A value that does not parse reads as 0, as extraction
// into a double leaves it.
bool read_named(const char *path, std::vector<std::string> &names, std::vector<double> &vals)
{
    std::ifstream in(path);
    if (!in.is_open()) return false;
    std::string line;
    while (std::getline(in, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream iss(line);
        std::string name;
        double v = 0;
        iss >> name >> v;
        names.push_back(name);
        vals.push_back(v);
    }
    return true;
}

// assign the named values to out[] by the key table; every key must appear
int assign(const char *what, const char *path, const char *const *keys, int nkeys,
           const std::vector<std::string> &names, const std::vector<double> &vals, double *out)
{
    std::vector<char> seen(nkeys, 0);
    for (size_t i = 0; i < names.size(); ++i) {
        int k = 0;
        while (k < nkeys && names[i] != keys[k]) ++k;
        if (k == nkeys)
            return fail(std::string(what) + ": unknown parameter '" + names[i] + "' in " + path);
        out[k] = vals[i];
        seen[k] = 1;
    }
    for (int k = 0; k < nkeys; ++k)
        if (!seen[k])
            return fail(std::string(what) + ": parameter '" + keys[k] + "' missing in " + path);
    return G3L_OK;
}

}  // namespace

namespace {

int g3l_read_function_impl(const char *path, double default_value, int nbins, double min, double max,
                      int log_bins, double *out)
{
    if (!path || !out || nbins < 1 || (log_bins && !(min > 0 && max > 0)))
        return fail("g3l_read_function: invalid arguments");
    std::ifstream in(path);
    if (!in.is_open()) return fail(std::string("g3l_read_function: cannot open ") + path);
    std::vector<double> xs, ys;
    double x, y;
    while (in >> x >> y) {
        xs.push_back(x);
        ys.push_back(y);
    }
    if (xs.empty()) return fail(std::string("g3l_read_function: no values in ") + path);
    if (log_bins) {
        const double bin = std::log(max / min) / nbins;
        for (int i = 0; i < nbins; ++i)
            out[i] = at_1d(xs, ys, std::exp(std::log(min) + i * bin), default_value);
    } else {
        const double bin = (max - min) / nbins;
        for (int i = 0; i < nbins; ++i) out[i] = at_1d(xs, ys, min + i * bin, default_value);
    }
    return G3L_OK;
}

int g3l_read_function2d_impl(const char *path, double default_value, int nbins, double min1,
                        double max1, double min2, double max2, double *out)
{
    if (!path || !out || nbins < 1 || !(min2 > 0 && max2 > 0))
        return fail("g3l_read_function2d: invalid arguments");
    std::ifstream in(path);
    if (!in.is_open()) return fail(std::string("g3l_read_function2d: cannot open ") + path);
    std::vector<double> ys;
    double x1, x2, y;
    while (in >> x1 >> x2 >> y) ys.push_back(y);
    if (ys.empty()) return fail(std::string("g3l_read_function2d: no values in ") + path);
    // the lookup with the grid set to the requested bins (src/Function2D.cpp:66-95)
    const int N = nbins;
    const double bin1 = (max1 - min1) / N;
    const double bin2 = std::log(max2 / min2) / N;
    for (int i = 0; i < N; ++i) {
        const double a = min1 + i * bin1;
        const int ix1 = (int)std::round((a - min1) * N / (max1 - min1));
        for (int j = 0; j < N; ++j) {
            const double b = std::exp(std::log(min2) + j * bin2);
            const int ix2 = (int)std::round(std::log(b / min2) * N / std::log(max2 / min2));
            double v = default_value;
            if (ix1 >= 0 && ix2 >= 0 && ix1 <= N && ix2 <= N) {
                const size_t idx = (size_t)ix1 * N + ix2;
                if (idx >= ys.size())
                    return fail(std::string("g3l_read_function2d: ") + path + " has " +
                                std::to_string(ys.size()) + " rows, fewer than the " +
                                std::to_string(N) + " x " + std::to_string(N) + " grid needs");
                v = ys[idx];
            }
            out[(size_t)i * N + j] = v;
        }
    }
    return G3L_OK;
}

int g3l_read_hod_params_impl(const char *path, double params[6])
{
    if (!path || !params) return fail("g3l_read_hod_params: invalid arguments");
    std::vector<std::string> names;
    std::vector<double> vals;
    if (!read_named(path, names, vals))
        return fail(std::string("g3l_read_hod_params: cannot open ") + path);
    // src/Params.cpp:38-63 keys, in the C ABI's order {f, alpha, Mth, sigma, M', beta}
    static const char *const keys[6] = {"f", "alpha", "M_min", "sigma", "M'", "beta"};
    return assign("g3l_read_hod_params", path, keys, 6, names, vals, params);
}

int g3l_read_cosmology_impl(const char *path, double cosmo[6])
{
    if (!path || !cosmo) return fail("g3l_read_cosmology: invalid arguments");
    std::vector<std::string> names;
    std::vector<double> vals;
    if (!read_named(path, names, vals))
        return fail(std::string("g3l_read_cosmology: cannot open ") + path);
    // src/Cosmology.cpp:36-68 keys
    static const char *const keys[6] = {"Omega_m", "Omega_Lambda", "Omega_b", "sigma8", "H0", "ns"};
    return assign("g3l_read_cosmology", path, keys, 6, names, vals, cosmo);
}

int g3l_read_triplets_impl(const char *path, double *thetas, int cap, int *n)
{
    if (!path || !n || cap < 0 || (cap > 0 && !thetas))
        return fail("g3l_read_triplets: invalid arguments");
    std::ifstream in(path);
    if (!in.is_open()) return fail(std::string("g3l_read_triplets: cannot open ") + path);
    int k = 0;
    double a, b, c;
    while (in >> a >> b >> c) {
        if (k < cap) {
            thetas[3 * k] = a;
            thetas[3 * k + 1] = b;
            thetas[3 * k + 2] = c;
        }
        ++k;
    }
    *n = k;
    return G3L_OK;
}

}  // namespace

// the C ABI: no exception crosses it (a file too large for host memory reports NOMEM)
extern "C" {

int g3l_read_function(const char *path, double default_value, int nbins, double min, double max, int log_bins, double *out)
{
    try {
        return g3l_read_function_impl(path, default_value, nbins, min, max, log_bins, out);
    } catch (const std::bad_alloc &) {
        return fail_nomem("g3l_read_function");
    }
}

int g3l_read_function2d(const char *path, double default_value, int nbins, double min1, double max1, double min2, double max2, double *out)
{
    try {
        return g3l_read_function2d_impl(path, default_value, nbins, min1, max1, min2, max2, out);
    } catch (const std::bad_alloc &) {
        return fail_nomem("g3l_read_function2d");
    }
}

int g3l_read_hod_params(const char *path, double params[6])
{
    try {
        return g3l_read_hod_params_impl(path, params);
    } catch (const std::bad_alloc &) {
        return fail_nomem("g3l_read_hod_params");
    }
}

int g3l_read_cosmology(const char *path, double cosmo[6])
{
    try {
        return g3l_read_cosmology_impl(path, cosmo);
    } catch (const std::bad_alloc &) {
        return fail_nomem("g3l_read_cosmology");
    }
}

int g3l_read_triplets(const char *path, double *thetas, int cap, int *n)
{
    try {
        return g3l_read_triplets_impl(path, thetas, cap, n);
    } catch (const std::bad_alloc &) {
        return fail_nomem("g3l_read_triplets");
    }
}

}  // extern "C"
