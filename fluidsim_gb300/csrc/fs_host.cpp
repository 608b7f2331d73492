// fs_host.cpp -- host-side set-up of the CUDA implementation: derived physical
// constants and the local-mean-energy coefficient table.
//
// Constants follow props.F90:24-47 and ptcl_props.F90:5-25.  Literals that the
// reference writes without a d exponent are REAL(4) in Fortran; they are
// rounded through float here (f32()).  Compiled with -ffp-contract=off so every
// product and sum is rounded separately, as in the Fortran.
#include <cmath>
#include <vector>

#include "fs_internal.h"

static inline double f32(float v) { return (double)v; }

void fs_host_constants(const fs_config &cfg, fs_constants &k) {
    k.pi = 4.0 * std::atan(1.0);
    k.eps0 = f32(8.85418782e-12f);
    k.e = f32(1.60217646e-19f);
    k.kb = f32(1.3806503e-23f);
    k.me = 9.10938188e-31;
    k.x0 = f32(1e-4f);
    k.ph0 = k.e / (k.eps0 * k.x0);
    k.t0 = f32(1e-6f);
    const double x03 = k.x0 * k.x0 * k.x0;
    k.wp02 = (k.t0 * k.t0) * (k.e * k.e) / (k.eps0 * x03 * k.me);
    k.w2 = (k.t0 * f32(14e9f)) * (k.t0 * f32(14e9f));
    k.tg = cfg.tg_k;
    k.p = cfg.p_torr;
    k.ninf = k.p * 101325.0 / 760.0 / k.kb / k.tg * x03;
    k.n_zero = f32(1e8f) * x03;
    k.mi = 1.67262178e-27 * 39.948;
    k.mui = 1.45e3 / k.p * 1e-4 * k.ph0 * k.t0 / (k.x0 * k.x0);
    k.vi = std::sqrt((8.0 * k.kb * k.tg) / (k.pi * k.mi)) * k.t0 / k.x0;
    k.Di = k.mui * (k.kb * k.tg / k.e) / k.ph0;
    k.Dm = 2.42e18 * k.x0 / k.ninf / 1e2 * k.t0;
    k.k_r = 2e-7 / 1e6 / x03 * k.t0;
    k.k_mp = 6.2e-10 / 1.0e6 / x03 * k.t0;
    k.k_2q = 3e-15 / 1e6 / x03 * k.t0;
    k.k_3q = 1.1e-31 / 1.0e12 / (x03 * x03) * k.t0;
    k.h_ir = 15.80 / k.ph0;
    k.h_ex = 11.56 / k.ph0;
    k.h_si = 4.14 / k.ph0;
    k.h_sc = -11.56 / k.ph0;
    k.gam = cfg.gam;
    k.nmin_nt = k.n_zero / k.ph0 / 1e2;
    k.cap = 1e-11 * k.ph0 / k.e;
}

// ---------------------------------------------------------------------------
// Coefficient fits of ptcl_props.F90:182-429 at nondimensional mean energy T,
// used to fill the table.  x**n with integer n is a multiplication chain.
namespace {
struct FitEval {
    double ph0, x0, t0, x03, ninf;
    static double q2(double x) { return x * x; }
    static double q3(double x) { return q2(x) * x; }
    static double q4(double x) { double t = q2(x); return t * t; }
    static double q5(double x) { return q3(x) * q2(x); }
    static double q6(double x) { double t = q3(x); return t * t; }
    static double q7(double x) { return q4(x) * q3(x); }
    static double q8(double x) { double t = q4(x); return t * t; }
    static double q9(double x) { return q6(x) * q3(x); }
    static double q10(double x) { double t = q5(x); return t * t; }
    static double q11(double x) { return q6(x) * q5(x); }
    double clog(double lo, double hi, double T) const { return std::log(std::max(lo, std::min(hi, T * ph0))); }

    double mue(double T) const {
        double x = clog(2.34e-1, 1.57e2, T), s;
        if (x < f32(std::log(5.119f)))
            s = f32(58.1133016145f) + f32(-0.984082217962f) * x + f32(-0.164770900119f) * q2(x)
              + f32(-0.142058042584f) * q3(x) + f32(-0.0637079234081f) * q4(x) + f32(0.0436642742558f) * q5(x);
        else
            s = f32(70.7846754548f) + f32(-22.7558138237f) * x + f32(12.8366493242f) * q2(x)
              + f32(-3.57242763244f) * q3(x) + f32(0.486276623664f) * q4(x) + f32(-0.0259045697422f) * q5(x);
        return std::exp(s) * x0 / ninf * t0 * ph0;
    }
    double De(double T) const {
        double x = clog(2.34e-1, 1.57e2, T);
        double s = f32(57.7067018813f) + f32(-0.0699892875381f) * x + f32(-0.117645585949f) * q2(x)
                 + f32(0.105390295278f) * q3(x) + f32(-0.102862612604f) * q4(x) + f32(-0.0469171521686f) * q5(x)
                 + f32(0.0584908312121f) * q6(x) + f32(0.000578601715687f) * q7(x) + f32(-0.0122860884883f) * q8(x)
                 + f32(0.00426793748856f) * q9(x) + f32(-0.000590000082557f) * q10(x) + f32(3.00706533201e-05f) * q11(x);
        return std::exp(s) * x0 / ninf * t0;
    }
    double k_ex(double T) const {
        double x = clog(9.611e-1, 1.57e2, T), s;
        if (x < f32(std::log(5.667f)))
            s = f32(-54.4513453969f) + f32(17.1472529739f) * x + f32(-1.05188982824f) * q2(x)
              + f32(-10.5053010711f) * q3(x) + f32(7.51502551486f) * q4(x) + f32(-1.44763942525f) * q5(x);
        else
            s = f32(-150.266369415f) + f32(158.67012941f) * x + f32(-85.5163470769f) * q2(x)
              + f32(23.0655081891f) * q3(x) + f32(-3.0908688844f) * q4(x) + f32(0.16403226902f) * q5(x);
        return std::exp(s) * t0 / x03;
    }
    double k_ir_fit(double T) const {
        double x = clog(1.37, 1.57e2, T), s;
        if (x < f32(std::log(7.5f)))
            s = f32(-73.27080258f) + f32(-30.1312514721f) * x + f32(138.743842326f) * q2(x)
              + f32(-161.378167125f) * q3(x) + f32(81.9325486193f) * q4(x) + f32(-14.9080865672f) * q5(x);
        else
            s = f32(-168.925304837f) + f32(177.113452524f) * x + f32(-92.3047166553f) * q2(x)
              + f32(24.1814225482f) * q3(x) + f32(-3.15463258104f) * q4(x) + f32(0.16331188192f) * q5(x);
        return std::exp(s) * t0 / x03;
    }
    double nu(double T) const {
        double x = clog(2.34e-1, 1.57e2, T);
        double s = f32(-32.275912575f) + f32(1.45173283977f) * x + f32(0.00936933121094f) * std::pow(x, 2.0)
                 + f32(0.129397015353f) * std::pow(x, 3.0) + f32(-0.0414865809044f) * std::pow(x, 4.0)
                 + f32(-0.0582934303409f) * std::pow(x, 5.0) + f32(0.0309832277826f) * std::pow(x, 6.0)
                 + f32(-0.00542014733763f) * q7(x) + f32(0.000325615321708f) * std::pow(x, 8.0);
        return std::exp(s) / x03 * ninf * t0;
    }
    double beta(double T) const {
        const double a = 11.604505e3;
        double x = std::log10(std::min(T * ph0 / 1.5 * a, 5e4));
        return std::pow(10.0, 0.944 - 0.665 * (x - f32(2.48f))) * 1e-13 * t0 / x03;
    }
    double k_sc(double T) const {
        double x = std::log(std::min(16.0, std::max(5e-1, T * ph0)));
        double s = f32(-21.4827864151f) + f32(0.457356923276f) * x + f32(-0.555439231606f) * std::pow(x, 2.0)
                 + f32(1.27257798891f) * std::pow(x, 3.0) + f32(-0.67840685073f) * std::pow(x, 4.0)
                 + f32(0.10591014464f) * std::pow(x, 5.0);
        return std::exp(s) / 1.0e6 / x03 * t0;
    }
    double k_si(double T) const {
        double x = std::log(std::min(16.0, std::max(5e-1, T * ph0)));
        double s = f32(-43.1347385848f) + f32(43.9905424566f) * x + f32(-28.1169537586f) * std::pow(x, 2.0)
                 + f32(8.28853856817f) * std::pow(x, 3.0) + f32(-0.931626144207f) * std::pow(x, 4.0);
        return std::exp(s) / 1.0e6 / x03 * t0;
    }
};
}  // namespace

// rows[r*n + k]: coefficient r (mue, De, k_ir, k_ex, nu, beta, k_sc, k_si) at
// mean energy eps_k = exp(ln emin + k h), h = ln(emax/emin)/(n-1), T = eps_k/ph0.
// k_ir is the Arrhenius rate A exp(-Ea/eps) [m^3/s] scaled by t0/x0**3.
void fs_host_table(const fs_config &cfg, const fs_constants &k, std::vector<double> &rows) {
    FitEval f;
    f.ph0 = k.ph0; f.x0 = k.x0; f.t0 = k.t0; f.x03 = k.x0 * k.x0 * k.x0; f.ninf = k.ninf;
    const int n = cfg.table_n;
    const double lemin = std::log(cfg.table_emin_ev), lemax = std::log(cfg.table_emax_ev);
    const double h = (lemax - lemin) / (double)(n - 1);
    rows.assign((size_t)8 * n, 0.0);
    for (int i = 0; i < n; i++) {
        double eps = std::exp(lemin + (double)i * h);
        double T = eps / k.ph0;
        rows[0 * (size_t)n + i] = f.mue(T);
        rows[1 * (size_t)n + i] = f.De(T);
        rows[2 * (size_t)n + i] = cfg.kir_arrh_a * std::exp(-cfg.kir_arrh_e / eps) * k.t0 / f.x03;
        rows[3 * (size_t)n + i] = f.k_ex(T);
        rows[4 * (size_t)n + i] = f.nu(T);
        rows[5 * (size_t)n + i] = f.beta(T);
        rows[6 * (size_t)n + i] = f.k_sc(T);
        rows[7 * (size_t)n + i] = f.k_si(T);
    }
}
