/*
 * g3lhalo_model.hpp -- the reference's model classes on the GB300 engine.
 *
 * Drop-in replacement for g3lhalo::NNMap_Model and g3lhalo::NMapMap_Model
 * (src/NNMap_Model.h:124-241, src/NMapMap_Model.h:102-169): same constructors, same
 * per-term methods and the same calculateAll, implemented over the C ABI of
 * libg3lgpu.so (g3l_gpu.h).  Include it in place of NNMap_Model.h / NMapMap_Model.h,
 * after the definitions of g3lhalo::Cosmology (fields Omega_m, Omega_Lambda, Omega_b,
 * sigma8, H0, ns; src/Cosmology.h:15-29) and g3lhalo::HOD (member `params` with f,
 * alpha, mmin, sigma, mprime, beta; src/HOD.h:22-28, src/Params.h:15-23), and link
 * -lg3lgpu.  Header-only; no CUDA headers are needed.
 *
 * Behaviour kept from the reference:
 *  - the per-term budgets: maxEval 5e6, rtol 1e-3 (NNMap 1h and 2h, every NMapMap
 *    term) or 1e-4 (NNMap 3h) (src/NNMap_Model.cu:318,343,368;
 *    src/NMapMap_Model.cu:186,211,236), and the prefactor chains;
 *  - type 1 / 2 select hod1 / hod2; the same-population satellite-pair branch is
 *    taken when both types name the same HOD object (src/HOD.cu:82);
 *  - calculateAll returns the N1N2, N1N1, N2N2 blocks in that order
 *    (src/NNMap_Model.cu:382-415); its A and epsilon arguments are applied here
 *    (the reference accepts but ignores them).
 * Differences:
 *  - errors do not exit(): a failing term returns NaN and lastStatus() / the C ABI's
 *    g3l_last_error() tell why;
 *  - the tables are copied to the device at construction (the reference also copies
 *    them; the caller's arrays need not outlive the model here);
 *  - the integrand runs in mixed precision by default (every term within 1e-4 of the
 *    all-FP64 form); setPrecision(G3L_FP64) selects the all-FP64 form;
 *  - calculateAll integrates every triplet and term in one device launch;
 *  - the SCALING constructor is always declared (the reference's needs -DSCALING,
 *    src/NNMap_Model.h:130-166); it copies scaling1 to the device for both HOD slots,
 *    which is what the reference computes (its same-population pair count reads only
 *    scaling1, src/NNMap_Model.cu:563,808, src/HOD.cu:86-87), and does not free() the
 *    caller's arrays as the reference's destructor does (src/NNMap_Model.cu:231-234).
 */
#ifndef G3LHALO_MODEL_HPP
#define G3LHALO_MODEL_HPP

#include <cmath>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "g3l_gpu.h"

namespace g3lhalo {

namespace gb300_detail {

inline void hod_params(const HOD *h, double out[6])
{
    out[0] = h->params->f;
    out[1] = h->params->alpha;
    out[2] = h->params->mmin;
    out[3] = h->params->sigma;
    out[4] = h->params->mprime;
    out[5] = h->params->beta;
}

// One engine context with the model's tables; HOD slots 0 (hod1) and 1 (hod2).
class Engine {
  public:
    Engine(const Cosmology *cosmo, double zmin, double zmax, double kmin, double kmax, double mmin,
           double mmax, int Nbins, const double *g, const double *p1, const double *p2,
           const double *w, const double *dwdz, const double *hmf, const double *P_lin,
           const double *b_h, const double *conc)
    {
        g3l_tables t{};
        t.Nz = t.Nm = t.Nk = Nbins;
        t.zmin = zmin;
        t.zmax = zmax;
        t.mmin = mmin;
        t.mmax = mmax;
        t.kmin = kmin;
        t.kmax = kmax;
        t.g = g;
        t.p_lens1 = p1;
        t.p_lens2 = p2;
        t.w = w;
        t.dwdz = dwdz;
        t.hmf = hmf;
        t.b_h = b_h;
        t.conc = conc;
        t.P_lin = P_lin;
        t.Om = cosmo->Omega_m;
        t.OL = cosmo->Omega_Lambda;
        t.Ob = cosmo->Omega_b;
        t.sigma8 = cosmo->sigma8;
        t.H0 = cosmo->H0;
        t.ns = cosmo->ns;
        t.clamp_k = 0;  // the reference's unclamped P_lin read
        if (g3l_ctx_create(&t, 0, &ctx_) != G3L_OK)
            throw std::runtime_error(std::string("g3lhalo GB300 engine: ") + g3l_last_error());
    }
    ~Engine() { g3l_ctx_destroy(ctx_); }
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;

    int setHOD(int slot, const HOD *h)
    {
        double p[6];
        hod_params(h, p);
        return g3l_set_hod(ctx_, slot, p);
    }
    int setCorrelation(double A, double eps) { return g3l_set_correlation(ctx_, A, eps); }

    // integrate items; returns the engine status, results in out
    int eval(const std::vector<g3l_integral> &items, std::vector<g3l_result> &out)
    {
        out.assign(items.size(), g3l_result{});
        if (items.empty()) return G3L_OK;
        return g3l_eval(ctx_, items.data(), (int)items.size(), precision, out.data());
    }

    g3l_ctx *ctx_ = nullptr;
    int precision = G3L_MIXED;
};

inline g3l_integral item(int kind, int term, int h1, int h2, double t1, double t2, double t3,
                         double rtol)
{
    g3l_integral it{};
    it.kind = kind;
    it.term = term;
    it.hod1 = h1;
    it.hod2 = h2;
    it.theta[0] = t1;
    it.theta[1] = t2;
    it.theta[2] = t3;
    it.rtol = rtol;
    it.max_eval = 5000000;
    return it;
}

}  // namespace gb300_detail

class NNMap_Model {
  public:
    NNMap_Model(Cosmology *cosmology_, const double &zmin_, const double &zmax_,
                const double &kmin_, const double &kmax_, const double &mmin_,
                const double &mmax_, const int &Nbins_, double *g_, double *p_lens1_,
                double *p_lens2_, double *w_, double *dwdz_, double *hmf_, double *P_lin_,
                double *b_h_, double *concentration_, HOD *hod1_, HOD *hod2_, double A_,
                double epsilon_)
        : cosmology(cosmology_), zmin(zmin_), zmax(zmax_), kmin(kmin_), kmax(kmax_),
          mmin(mmin_), mmax(mmax_), Nbins(Nbins_), A(A_), epsilon(epsilon_),
          eng_(cosmology_, zmin_, zmax_, kmin_, kmax_, mmin_, mmax_, Nbins_, g_, p_lens1_,
               p_lens2_, w_, dwdz_, hmf_, P_lin_, b_h_, concentration_)
    {
        eng_.setCorrelation(A_, epsilon_);
        updateHODs(hod1_, hod2_);
    }

    /// The reference's SCALING constructor (src/NNMap_Model.cu:103-200): satellite-
    /// variance rescaling per mass bin, [Nbins] each
    NNMap_Model(Cosmology *cosmology_, const double &zmin_, const double &zmax_,
                const double &kmin_, const double &kmax_, const double &mmin_,
                const double &mmax_, const int &Nbins_, double *g_, double *p_lens1_,
                double *p_lens2_, double *w_, double *dwdz_, double *hmf_, double *P_lin_,
                double *b_h_, double *concentration_, double *scaling1_, double *scaling2_,
                HOD *hod1_, HOD *hod2_, double A_, double epsilon_)
        : NNMap_Model(cosmology_, zmin_, zmax_, kmin_, kmax_, mmin_, mmax_, Nbins_, g_, p_lens1_,
                      p_lens2_, w_, dwdz_, hmf_, P_lin_, b_h_, concentration_, hod1_, hod2_, A_,
                      epsilon_)
    {
        scaling1 = scaling1_;
        scaling2 = scaling2_;
        if (!status_) status_ = g3l_set_scaling(eng_.ctx_, 0, scaling1_);
        if (!status_) status_ = g3l_set_scaling(eng_.ctx_, 1, scaling1_);
    }

    /// New HODs: recomputes n_bar(z) for both (src/NNMap_Model.cu:244-297)
    void updateHODs(HOD *hod1_, HOD *hod2_)
    {
        hod1 = hod1_;
        hod2 = hod2_;
        status_ = eng_.setHOD(0, hod1_);
        if (!status_) status_ = eng_.setHOD(1, hod2_);
    }

    double NNMap_1h(const double &theta1, const double &theta2, const double &theta3,
                    const int &type1, const int &type2)
    {
        return term(1, 1e-3, theta1, theta2, theta3, type1, type2);
    }
    double NNMap_2h(const double &theta1, const double &theta2, const double &theta3,
                    const int &type1, const int &type2)
    {
        return term(2, 1e-3, theta1, theta2, theta3, type1, type2);
    }
    double NNMap_3h(const double &theta1, const double &theta2, const double &theta3,
                    const int &type1, const int &type2)
    {
        return term(3, 1e-4, theta1, theta2, theta3, type1, type2);
    }
    /// Sum of the three terms, integrated together in one launch
    double NNMap(const double &theta1, const double &theta2, const double &theta3,
                 const int &type1, const int &type2)
    {
        std::vector<g3l_integral> items;
        for (int t = 1; t <= 3; ++t)
            items.push_back(gb300_detail::item(G3L_NNMAP, t, slot(type1), slot(type2), theta1,
                                               theta2, theta3, t == 3 ? 1e-4 : 1e-3));
        std::vector<g3l_result> r;
        status_ = eng_.eval(items, r);
        if (status_) return std::numeric_limits<double>::quiet_NaN();
        return r[0].result + r[1].result + r[2].result;
    }

    /// All triplets, N1N2 then N1N1 then N2N2, in one launch
    void calculateAll(const std::vector<double> &thetas1, const std::vector<double> &thetas2,
                      const std::vector<double> &thetas3, HOD *hod1_, HOD *hod2_, double A_,
                      double epsilon_, std::vector<double> &results)
    {
        A = A_;
        epsilon = epsilon_;
        eng_.setCorrelation(A_, epsilon_);
        updateHODs(hod1_, hod2_);
        const int pairs[3][2] = {{1, 2}, {1, 1}, {2, 2}};
        const size_t n = thetas1.size();
        std::vector<g3l_integral> items;
        for (const auto &pr : pairs)
            for (size_t i = 0; i < n; ++i)
                for (int t = 1; t <= 3; ++t)
                    items.push_back(gb300_detail::item(G3L_NNMAP, t, slot(pr[0]), slot(pr[1]),
                                                       thetas1.at(i), thetas2.at(i),
                                                       thetas3.at(i), t == 3 ? 1e-4 : 1e-3));
        std::vector<g3l_result> r;
        status_ = eng_.eval(items, r);
        for (size_t k = 0; k < items.size(); k += 3)
            results.push_back(status_ ? std::numeric_limits<double>::quiet_NaN()
                                      : r[k].result + r[k + 1].result + r[k + 2].result);
    }

    /// G3L_MIXED (default) or G3L_FP64
    void setPrecision(int precision) { eng_.precision = precision; }
    /// Status of the last call (G3L_OK = 0); g3l_last_error() has the message
    int lastStatus() const { return status_; }
    g3l_ctx *context() { return eng_.ctx_; }

    Cosmology *cosmology;
    double zmin, zmax, kmin, kmax, mmin, mmax;
    int Nbins;
    double A, epsilon;
    HOD *hod1 = nullptr, *hod2 = nullptr;
    double *scaling1 = nullptr, *scaling2 = nullptr;  // SCALING constructor only

  private:
    // type 1 -> slot 0, type 2 -> slot 1; one HOD object for both types -> one slot,
    // so the same-population branch follows the object, as in the reference
    int slot(int type) const { return (type == 2 && hod2 != hod1) ? 1 : 0; }

    double term(int t, double rtol, double t1, double t2, double t3, int type1, int type2)
    {
        std::vector<g3l_result> r;
        status_ = eng_.eval({gb300_detail::item(G3L_NNMAP, t, slot(type1), slot(type2), t1, t2, t3,
                                                rtol)},
                            r);
        return status_ ? std::numeric_limits<double>::quiet_NaN() : r[0].result;
    }

    gb300_detail::Engine eng_;
    int status_ = G3L_OK;
};

class NMapMap_Model {
  public:
    NMapMap_Model(Cosmology *cosmology_, const double &zmin_, const double &zmax_,
                  const double &kmin_, const double &kmax_, const double &mmin_,
                  const double &mmax_, const int &Nbins_, double *g_, double *p_lens_,
                  double *w_, double *dwdz_, double *hmf_, double *P_lin_, double *b_h_,
                  double *concentration_, HOD *hod_)
        : cosmology(cosmology_), zmin(zmin_), zmax(zmax_), kmin(kmin_), kmax(kmax_),
          mmin(mmin_), mmax(mmax_), Nbins(Nbins_),
          eng_(cosmology_, zmin_, zmax_, kmin_, kmax_, mmin_, mmax_, Nbins_, g_, p_lens_, p_lens_,
               w_, dwdz_, hmf_, P_lin_, b_h_, concentration_)
    {
        updateHOD(hod_);
    }

    void updateHOD(HOD *hod_)
    {
        hod = hod_;
        status_ = eng_.setHOD(0, hod_);
    }

    double NMapMap_1h(const double &theta1, const double &theta2, const double &theta3)
    {
        return term(1, theta1, theta2, theta3);
    }
    double NMapMap_2h(const double &theta1, const double &theta2, const double &theta3)
    {
        return term(2, theta1, theta2, theta3);
    }
    double NMapMap_3h(const double &theta1, const double &theta2, const double &theta3)
    {
        return term(3, theta1, theta2, theta3);
    }
    double NMapMap(const double &theta1, const double &theta2, const double &theta3)
    {
        std::vector<g3l_integral> items;
        for (int t = 1; t <= 3; ++t)
            items.push_back(gb300_detail::item(G3L_NMAPMAP, t, 0, 0, theta1, theta2, theta3, 1e-3));
        std::vector<g3l_result> r;
        status_ = eng_.eval(items, r);
        if (status_) return std::numeric_limits<double>::quiet_NaN();
        return r[0].result + r[1].result + r[2].result;
    }

    void calculateAll(const std::vector<double> &thetas1, const std::vector<double> &thetas2,
                      const std::vector<double> &thetas3, HOD *hod_, std::vector<double> &results)
    {
        updateHOD(hod_);
        std::vector<g3l_integral> items;
        for (size_t i = 0; i < thetas1.size(); ++i)
            for (int t = 1; t <= 3; ++t)
                items.push_back(gb300_detail::item(G3L_NMAPMAP, t, 0, 0, thetas1.at(i),
                                                   thetas2.at(i), thetas3.at(i), 1e-3));
        std::vector<g3l_result> r;
        status_ = eng_.eval(items, r);
        for (size_t k = 0; k < items.size(); k += 3)
            results.push_back(status_ ? std::numeric_limits<double>::quiet_NaN()
                                      : r[k].result + r[k + 1].result + r[k + 2].result);
    }

    void setPrecision(int precision) { eng_.precision = precision; }
    int lastStatus() const { return status_; }
    g3l_ctx *context() { return eng_.ctx_; }

    Cosmology *cosmology;
    double zmin, zmax, kmin, kmax, mmin, mmax;
    int Nbins;
    HOD *hod = nullptr;

  private:
    double term(int t, double t1, double t2, double t3)
    {
        std::vector<g3l_result> r;
        status_ = eng_.eval({gb300_detail::item(G3L_NMAPMAP, t, 0, 0, t1, t2, t3, 1e-3)}, r);
        return status_ ? std::numeric_limits<double>::quiet_NaN() : r[0].result;
    }

    gb300_detail::Engine eng_;
    int status_ = G3L_OK;
};

}  // namespace g3lhalo

#endif /* G3LHALO_MODEL_HPP */
