// Runs the reference's model interface (g3lhalo_model.hpp) on tables read from a
// binary file and prints one "name value" line per result.
//
// File layout (little-endian): int32 N; float64 zmin zmax kmin kmax mmin mmax;
// cosmology[6] (Om, OL, Ob, sigma8, H0, ns); hod1[6]; hod2[6] (f, alpha, Mth, sigma,
// M', beta); g, p_lens1, p_lens2, w, dwdz [N]; hmf, P_lin, b_h, concentration [N*N];
// thetas[4][3] (rad); with argv[3] = 1 also scaling1, scaling2 [N], for the SCALING
// constructor.  argv[2]: 0 = all-FP64 form, 1 = mixed precision.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "shim_types.h"
#include "g3lhalo_model.hpp"

int main(int argc, char **argv)
{
    if (argc < 3) return 2;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    int N = 0;
    double bin[6], cos[6], h1[6], h2[6];
    bool ok = std::fread(&N, 4, 1, f) == 1 && std::fread(bin, 8, 6, f) == 6 &&
              std::fread(cos, 8, 6, f) == 6 && std::fread(h1, 8, 6, f) == 6 &&
              std::fread(h2, 8, 6, f) == 6;
    std::vector<std::vector<double>> v1(5, std::vector<double>(N)), v2(4, std::vector<double>(N * N));
    for (auto &a : v1) ok = ok && std::fread(a.data(), 8, N, f) == (size_t)N;
    for (auto &a : v2) ok = ok && std::fread(a.data(), 8, (size_t)N * N, f) == (size_t)N * N;
    double th[4][3];
    ok = ok && std::fread(th, 8, 12, f) == 12;
    const bool scaled = argc > 3 && std::atoi(argv[3]) == 1;
    std::vector<double> s1(N), s2(N);
    if (scaled)
        ok = ok && std::fread(s1.data(), 8, N, f) == (size_t)N &&
             std::fread(s2.data(), 8, N, f) == (size_t)N;
    std::fclose(f);
    if (!ok) return 4;
    g3lhalo::Cosmology c;
    c.Omega_m = cos[0];
    c.Omega_Lambda = cos[1];
    c.Omega_b = cos[2];
    c.sigma8 = cos[3];
    c.H0 = cos[4];
    c.ns = cos[5];
    auto params = [](const double *p) {
        g3lhalo::Params q;
        q.f = p[0];
        q.alpha = p[1];
        q.mmin = p[2];
        q.sigma = p[3];
        q.mprime = p[4];
        q.beta = p[5];
        return q;
    };
    g3lhalo::Params p1 = params(h1), p2 = params(h2);
    g3lhalo::HOD hod1(&p1), hod2(&p2);
    const int prec = std::atoi(argv[2]) ? G3L_MIXED : G3L_FP64;

    if (scaled) {  // the SCALING constructor; same-population terms
        g3lhalo::NNMap_Model ns(&c, bin[0], bin[1], bin[2], bin[3], bin[4], bin[5], N,
                                v1[0].data(), v1[1].data(), v1[2].data(), v1[3].data(),
                                v1[4].data(), v2[0].data(), v2[1].data(), v2[2].data(),
                                v2[3].data(), s1.data(), s2.data(), &hod1, &hod2, 0.0, 0.0);
        ns.setPrecision(prec);
        std::printf("S_NNMap_1h %.17g\n", ns.NNMap_1h(th[1][0], th[1][1], th[1][2], 1, 1));
        std::printf("S_NNMap_2h %.17g\n", ns.NNMap_2h(th[1][0], th[1][1], th[1][2], 1, 1));
        std::printf("status %d\n", ns.lastStatus());
        return 0;
    }

    g3lhalo::NNMap_Model nn(&c, bin[0], bin[1], bin[2], bin[3], bin[4], bin[5], N, v1[0].data(),
                            v1[1].data(), v1[2].data(), v1[3].data(), v1[4].data(), v2[0].data(),
                            v2[1].data(), v2[2].data(), v2[3].data(), &hod1, &hod2, 0.0, 0.0);
    nn.setPrecision(prec);
    std::printf("NNMap_1h %.17g\n", nn.NNMap_1h(th[1][0], th[1][1], th[1][2], 1, 2));
    std::printf("NNMap_2h %.17g\n", nn.NNMap_2h(th[1][0], th[1][1], th[1][2], 1, 2));
    std::printf("NNMap_3h %.17g\n", nn.NNMap_3h(th[1][0], th[1][1], th[1][2], 1, 2));
    std::printf("NNMap %.17g\n", nn.NNMap(th[1][0], th[1][1], th[1][2], 1, 2));
    std::vector<double> t1, t2, t3, res;
    for (int i = 0; i < 2; ++i) {
        t1.push_back(th[i][0]);
        t2.push_back(th[i][1]);
        t3.push_back(th[i][2]);
    }
    nn.calculateAll(t1, t2, t3, &hod1, &hod2, 0.0, 0.0, res);
    for (size_t i = 0; i < res.size(); ++i) std::printf("calculateAll_%zu %.17g\n", i, res[i]);
    std::printf("status %d\n", nn.lastStatus());

    g3lhalo::NMapMap_Model nm(&c, bin[0], bin[1], bin[2], bin[3], bin[4], bin[5], N, v1[0].data(),
                              v1[1].data(), v1[3].data(), v1[4].data(), v2[0].data(), v2[1].data(),
                              v2[2].data(), v2[3].data(), &hod2);
    nm.setPrecision(prec);
    std::printf("NMapMap_1h %.17g\n", nm.NMapMap_1h(th[0][0], th[0][1], th[0][2]));
    std::printf("status %d\n", nm.lastStatus());
    return 0;
}
