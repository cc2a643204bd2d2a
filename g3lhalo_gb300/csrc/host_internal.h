// host_internal.h -- host-side helpers shared by the library's translation units.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "g3l_gpu.h"

namespace g3l {
namespace host {

void set_error(const std::string &msg);

int cubature(unsigned dim, g3l_integrand_v f, void *fdata, const double *xmin, const double *xmax,
             size_t maxEval, double reqAbs, double reqRel, double *val, double *err,
             size_t *neval);

// Binning and integration bounds of the reference (src/NNMap_Model.cu:46-49,313-314).
struct Binning {
    int Nz, Nm, Nk;
    double zmin, zmax, mmin, mmax, kmin, kmax;
    double mmax_integral() const;
    double zmax_integral() const;
    // xmin/xmax of a term (dim = term + 4); returns dim
    int bounds(int term, double *xmin, double *xmax) const;
};

// rho_bar(z_i) = Omega_m(z) rho_crit (src/NNMap_Model.cu:256, src/Cosmology.cpp:71-87)
void rho_bar(const Binning &B, double Om, double OL, double H0, double *out);
// n_bar(z_i) for one HOD (src/NNMap_Model.cu:244-297, src/generalFunctions.cu:149-245)
int n_bar(const Binning &B, const double *hmf, const double hod[6], double *out);
// n_bar(z_i) on the device (precompute.cu): device buffers a context keeps between calls
struct NbarDevice {
    void *tasks = nullptr, *out = nullptr, *idx = nullptr, *cache = nullptr;
    double *hods = nullptr;
    size_t ntask_cap = 0, nhod_cap = 0;
};
void free_nbar_device(NbarDevice &W);
// n_bar(z_i) of nh HOD vectors (hods: [nh][6] on the host) on the current device from its
// FP64 mass function d_hmf [Nz][Nm]; out: [nh][Nz] on the host.  stream: a cudaStream_t.
int n_bar_device(NbarDevice &W, const Binning &B, const double *d_hmf, const double *hods,
                 int nh, void *stream, int nsm, double *out);
// the reference's prefactor chain applied to a raw integral
double apply_prefactor(int kind, int term, double H0, double Om, double raw);

// exact m indices of the tie-prone centre values (sorted by bit pattern)
struct TieTable {
    std::vector<unsigned long long> bits;
    std::vector<int> round_ix, trunc_ix;
};
TieTable build_m_ties(const Binning &B);
TieTable build_z_ties(const Binning &B);

}  // namespace host
}  // namespace g3l
