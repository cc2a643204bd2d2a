// Minimal stand-ins for the reference's Cosmology, Params and HOD classes, with the
// fields g3lhalo_model.hpp reads (the reference's own classes carry more).  They let
// the C++ shim be built and run where the reference sources are not available.
#pragma once

namespace g3lhalo {

class Cosmology {
  public:
    double Omega_m = 0, Omega_Lambda = 0, Omega_b = 0, sigma8 = 0, H0 = 0, ns = 0;
};

class Params {
  public:
    double f = 1, alpha = 1, mmin = 1e12, sigma = 0.3, mprime = 1e13, beta = 1;
};

class HOD {
  public:
    explicit HOD(Params *p) : params(p) {}
    Params *params;
};

}  // namespace g3lhalo
