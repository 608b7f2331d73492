// fs_host.cpp -- host-side set-up of the CUDA implementation: derived physical
// constants and the local-mean-energy coefficient table.
//
// Constants follow props.F90:24-47 and ptcl_props.F90:5-25.  Literals that the
// reference writes without a d exponent are REAL(4) in Fortran; they are
// rounded through float here (f32()).  Compiled with -ffp-contract=off so every
// product and sum is rounded separately, as in the Fortran.
#include <cmath>
#include <vector>

#include "fs_fits.h"
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


// rows[r*n + k]: coefficient r (mue, De, k_ir, k_ex, nu, beta, k_sc, k_si) at
// mean energy eps_k = exp(ln emin + k h), h = ln(emax/emin)/(n-1), T = eps_k/ph0.
// k_ir is the Arrhenius rate A exp(-Ea/eps) [m^3/s] scaled by t0/x0**3.
FitEval fs_fit_eval(const fs_constants &k) {
    FitEval f;
    f.ph0 = k.ph0; f.x0 = k.x0; f.t0 = k.t0; f.x03 = k.x0 * k.x0 * k.x0; f.ninf = k.ninf;
    f.th_mue = f32(std::log(5.119f));
    f.th_kex = f32(std::log(5.667f));
    f.th_kir = f32(std::log(7.5f));
    return f;
}

void fs_host_table(const fs_config &cfg, const fs_constants &k, std::vector<double> &rows) {
    const FitEval f = fs_fit_eval(k);
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

// Source voltage of circ_step (circ_lib.F90:26-50) at nondimensional time t:
// DC, AC sin(pi t) (a 2 us period), and the two pulse shapes.  x**3 and x**2
// are products, as gfortran evaluates integer powers.
double fs_circ_source(const fs_config &cfg, const fs_constants &k, double t) {
    const double pi = k.pi, V = cfg.vl;
    switch (cfg.rf) {
    case 1: return V * std::sin(pi * t);
    case 2:
        if (t < 2.5e-1) { double s = std::sin(4 * pi * t); return V * (s * s * s); }
        return 0.0;
    case 3:
        if (t < 2.3e-1) { double s = std::sin(4.0 * pi * t); return V * (s * s); }
        if (t < 3.35e-1) return V * (std::sin(3.81 * pi * (t + 5.85e-2)) * 7.19e-1 + 2.81e-1);
        if (t < 8.2e-1) { double s = std::sin(3.81 * pi * (t + 1.2e-1) / 3.5); return V * ((s * s * s) * (-4.38e-1)); }
        return 0.0;
    default: return V;
    }
}
