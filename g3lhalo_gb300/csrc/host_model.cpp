// host_model.cpp -- host parts of the model: binning, densities, prefactors, tie table.
//
// Everything here runs once per table set or per HOD vector, in FP64 with the
// reference's expressions (compiled with -ffp-contract=off), so that rho_bar,
// n_bar and the integration bounds equal the reference's bit for bit on the
// same libm.
#include <algorithm>
#include <atomic>
#include <memory>
#include <thread>
#include <vector>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <system_error>

#include "host_internal.h"

namespace g3l {
namespace host {

namespace {
thread_local std::string g_last_error;
constexpr double kPi = 3.14159;          // truncated pi (src/constants.h:15)
constexpr double kC = 2.99792e5;         // km/s (src/constants.h:39)
constexpr double kMpcInKm = 3.086e19;    // src/Cosmology.h:28
constexpr double kG = 1.327e11;          // src/Cosmology.h:27
}  // namespace

void set_error(const std::string &msg) { g_last_error = msg; }
const char *last_error_cstr() { return g_last_error.c_str(); }

double Binning::mmax_integral() const
{
    return std::exp(std::log(mmin) + std::log(mmax / mmin) * (Nm - 1) / Nm);
}
double Binning::zmax_integral() const { return zmax - (zmax - zmin) / Nz; }

int Binning::bounds(int term, double *xmin, double *xmax) const
{
    const double lm0 = std::log10(mmin), lm1 = std::log10(mmax_integral());
    int d = 0;
    xmin[d] = std::log10(0.1); xmax[d++] = std::log10(1e6);
    xmin[d] = std::log10(0.1); xmax[d++] = std::log10(1e6);
    xmin[d] = 0; xmax[d++] = 2 * kPi;
    for (int j = 0; j < term; ++j) {
        xmin[d] = lm0;
        xmax[d++] = lm1;
    }
    xmin[d] = zmin;
    xmax[d++] = zmax_integral();
    return d;
}

void rho_bar(const Binning &B, double Om, double OL, double H0, double *out)
{
    const double rho_crit = 3 * H0 * H0 * kMpcInKm / 8 / kPi / kG;
    for (int i = 0; i < B.Nz; ++i) {
        double z = B.zmin + i * (B.zmax - B.zmin) / B.Nz;
        double E = Om * (1 + z) * (1 + z) * (1 + z) + OL;
        out[i] = Om * (1 + z) * (1 + z) * (1 + z) / E * rho_crit;
    }
}

namespace {
// The mass-dependent factors of the n_bar integrand (m, N_c + N_s and the mass bin)
// do not depend on z, and the 1-D Gauss-Kronrod regions of the Nz integrals come from
// bisecting the same interval, so most 15-point blocks recur in many z bins (a
// 64 x 128 table set evaluates ~1.5M points per HOD vector at ~30k distinct
// abscissae).  A table shared by the worker threads keeps each block's factors;
// every value is computed by the same expression as without the table, so n_bar is
// unchanged to the last bit.  A slot is claimed by CAS and published with a release
// store; a reader that meets a slot being filled computes its block itself.
constexpr int kGK = 15;  // points per 1-D region

struct BlockFactors {
    double x[kGK], m[kGK], S[kGK];  // abscissae, m, N_c + N_s
    int mix[kGK];                   // nearest mass bin
};

class BlockCache {
   public:
    explicit BlockCache(int log2cap)
        : cap_(1u << log2cap), shift_(64 - log2cap), st_(new std::atomic<unsigned>[cap_]()),
          dat_(new BlockFactors[cap_])
    {
    }
    // factors of the block at x[0..14]: from the table, or computed by fill() and
    // (if a slot is free) stored
    template <class Fill>
    const BlockFactors *get(const double *x, BlockFactors &local, Fill fill)
    {
        unsigned long long k0, k1;
        std::memcpy(&k0, x, 8);
        std::memcpy(&k1, x + 1, 8);
        unsigned idx = (unsigned)(((k0 * 0x9E3779B97F4A7C15ull) ^ (k1 * 0xC2B2AE3D27D4EB4Full)) >> shift_);
        for (int probe = 0; probe < 32; ++probe, idx = (idx + 1) & (cap_ - 1)) {
            unsigned s = st_[idx].load(std::memory_order_acquire);
            if (s == 0) {
                if (used_.load(std::memory_order_relaxed) >= cap_ / 4 * 3) break;
                if (st_[idx].compare_exchange_strong(s, 1u, std::memory_order_acq_rel)) {
                    used_.fetch_add(1, std::memory_order_relaxed);
                    BlockFactors &b = dat_[idx];
                    fill(x, b);
                    st_[idx].store(2u, std::memory_order_release);
                    return &b;
                }
            }
            if (s == 1) break;  // being filled: compute this block here
            if (s == 2 && std::memcmp(dat_[idx].x, x, sizeof(double) * kGK) == 0) return &dat_[idx];
        }
        fill(x, local);
        return &local;
    }

   private:
    unsigned cap_, shift_;
    std::unique_ptr<std::atomic<unsigned>[]> st_;
    std::unique_ptr<BlockFactors[]> dat_;
    std::atomic<unsigned> used_{0};
};

struct NbarCtx {
    const Binning *B;
    const double *hmf;
    const double *hod;  // f, alpha, Mth, sigma, M', beta
    double z;
    BlockCache *cache;
};

// N_c, N_s (src/HOD.cu:35-76) and the mass bin (src/NNMap_Model.cu:556) at x = log10 m;
// erf is evaluated once for both occupations (the same argument in the reference)
inline void mass_factors(const Binning &B, const double *h, double x, double &m, double &S,
                         int &mix)
{
    m = std::pow(10, x);
    const double e = std::erf(std::log(m / h[2]) / h[3] / 1.414213562);
    const double Nc = 0.5 * h[1] * (1 + e);
    const double Ns = 0.5 * (1 + e) * std::pow(m / h[4], h[5]);
    S = Nc + Ns;
    mix = (int)std::round(std::log(m / B.mmin) * B.Nm / std::log(B.mmax / B.mmin));
}

// ln10 m n(m, z) (N_c + N_s) without the ln10 (src/NNMap_Model.cu:262-297,
// src/generalFunctions.cu:233-245)
int nbar_integrand(unsigned ndim, size_t npt, const double *x, void *fdata, unsigned, double *fv)
{
    const NbarCtx *C = (const NbarCtx *)fdata;
    const Binning &B = *C->B;
    const double *h = C->hod;
    const int z_ix = (int)std::round((C->z - B.zmin) * B.Nz / (B.zmax - B.zmin));
    const double *row = C->hmf + (size_t)z_ix * B.Nm;
    if (ndim == 1 && npt % kGK == 0) {
        auto fill = [&](const double *xb, BlockFactors &b) {
            for (int k = 0; k < kGK; ++k) {
                b.x[k] = xb[k];
                mass_factors(B, h, xb[k], b.m[k], b.S[k], b.mix[k]);
            }
        };
        BlockFactors local;
        for (size_t i = 0; i < npt; i += kGK) {
            const BlockFactors *b = C->cache->get(x + i, local, fill);
            for (int k = 0; k < kGK; ++k) fv[i + k] = b->m[k] * row[b->mix[k]] * b->S[k];
        }
        return 0;
    }
    for (size_t i = 0; i < npt; ++i) {
        double m, S;
        int mix;
        mass_factors(B, h, x[i * ndim], m, S, mix);
        fv[i] = m * row[mix] * S;
    }
    return 0;
}
}  // namespace

int n_bar(const Binning &B, const double *hmf, const double hod[6], double *out)
{
    const double lo[1] = {std::log10(B.mmin)};
    const double hi[1] = {std::log10(B.mmax_integral())};
    const double ln10 = std::log(10.0);
    BlockCache cache(13);
    // the Nz integrals are independent: spread them over the host cores (each one is
    // the same sequential computation as in a single thread)
    std::atomic<int> next{0}, failed{0};
    auto work = [&]() {
        for (int i; (i = next.fetch_add(1)) < B.Nz;) {
            NbarCtx C{&B, hmf, hod, B.zmin + i * (B.zmax - B.zmin) / B.Nz, &cache};
            double val, err;
            if (cubature(1, nbar_integrand, &C, lo, hi, 0, 0, 1e-4, &val, &err, nullptr)) {
                failed = 1;
                continue;
            }
            out[i] = ln10 * val;
        }
    };
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int nt = (int)std::min<unsigned>(hw, (unsigned)std::max(1, B.Nz / 2));
    std::vector<std::thread> pool;
    pool.reserve(nt);
    for (int t = 1; t < nt; ++t) {
        try {
            pool.emplace_back(work);
        } catch (const std::system_error &) {
            break;  // fewer threads: the work loop takes what is left
        }
    }
    work();
    for (auto &th : pool) th.join();
    return failed.load() ? 1 : 0;
}

double apply_prefactor(int kind, int term, double H0, double Om, double raw)
{
    const double l10 = std::log(10.0);
    double r;
    if (kind == 0) r = raw * 3 * H0 * H0 * Om / 2 / kC / kC;
    else r = raw * 9 * std::pow(H0, 4) * std::pow(Om, 2) / 4 / std::pow(kC, 4);
    for (int i = 0; i < term + 2; ++i) r = r * l10;
    return r / (2 * kPi) / (2 * kPi) / (2 * kPi);
}

// Region centres along a mass dimension are reached by repeated exact bisection of
// [log10 mmin, log10 mmax_integral]; at depth L the centre sits at (2i+1)/2^(L+1) of
// the range, i.e. at index argument (2i+1)(Nm-1)/2^(L+1).  With Nm-1 = 2^a b (b odd)
// that argument is a half-integer (a tie of round()) at L = a and an integer (a tie
// of the truncation) at L < a.  Those centres are enumerated with the same FP64
// operations as the cut, and their indices evaluated with the reference's own
// expression on this host.
TieTable build_m_ties(const Binning &B)
{
    TieTable T;
    int a = 0;
    for (int v = B.Nm - 1; v > 0 && !(v & 1); v >>= 1) ++a;
    if (a > 12) a = 12;
    const double lo = std::log10(B.mmin), hi = std::log10(B.mmax_integral());
    struct Node { double c; int L; };
    std::vector<Node> stack{{0.5 * (lo + hi), 0}};
    const double hw0 = 0.5 * (hi - lo);
    std::vector<std::pair<unsigned long long, std::pair<int, int>>> rows;
    while (!stack.empty()) {
        Node nd = stack.back();
        stack.pop_back();
        double m = std::pow(10, nd.c);
        double arg = std::log(m / B.mmin) * B.Nm / std::log(B.mmax / B.mmin);
        unsigned long long bits;
        std::memcpy(&bits, &nd.c, sizeof bits);
        rows.push_back({bits, {(int)std::round(arg), (int)arg}});
        if (nd.L < a) {
            double hwc = std::ldexp(hw0, -(nd.L + 1));
            stack.push_back({nd.c - hwc, nd.L + 1});
            stack.push_back({nd.c + hwc, nd.L + 1});
        }
    }
    std::sort(rows.begin(), rows.end());
    rows.erase(std::unique(rows.begin(), rows.end(),
                           [](const auto &x, const auto &y) { return x.first == y.first; }),
               rows.end());
    for (auto &r : rows) {
        T.bits.push_back(r.first);
        T.round_ix.push_back(r.second.first);
        T.trunc_ix.push_back(r.second.second);
    }
    return T;
}

// The same enumeration for the redshift axis [zmin, zmax_integral]; its index
// arguments (z - zmin) Nz / (zmax - zmin) are exact FP64 expressions.
TieTable build_z_ties(const Binning &B)
{
    TieTable T;
    int a = 0;
    for (int v = B.Nz - 1; v > 0 && !(v & 1); v >>= 1) ++a;
    if (a > 12) a = 12;
    const double lo = B.zmin, hi = B.zmax_integral();
    struct Node { double c; int L; };
    std::vector<Node> stack{{0.5 * (lo + hi), 0}};
    const double hw0 = 0.5 * (hi - lo);
    std::vector<std::pair<unsigned long long, std::pair<int, int>>> rows;
    while (!stack.empty()) {
        Node nd = stack.back();
        stack.pop_back();
        double arg = (nd.c - B.zmin) * B.Nz / (B.zmax - B.zmin);
        unsigned long long bits;
        std::memcpy(&bits, &nd.c, sizeof bits);
        rows.push_back({bits, {(int)std::round(arg), (int)arg}});
        if (nd.L < a) {
            double hwc = std::ldexp(hw0, -(nd.L + 1));
            stack.push_back({nd.c - hwc, nd.L + 1});
            stack.push_back({nd.c + hwc, nd.L + 1});
        }
    }
    std::sort(rows.begin(), rows.end());
    rows.erase(std::unique(rows.begin(), rows.end(),
                           [](const auto &x, const auto &y) { return x.first == y.first; }),
               rows.end());
    for (auto &r : rows) {
        T.bits.push_back(r.first);
        T.round_ix.push_back(r.second.first);
        T.trunc_ix.push_back(r.second.second);
    }
    return T;
}

}  // namespace host
}  // namespace g3l
