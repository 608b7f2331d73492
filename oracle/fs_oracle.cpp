// fs_oracle.cpp -- CPU oracle of the fluidsim hot path (TEST INFRASTRUCTURE).
//
// A restatement of the reference Fortran in C++, routine by routine and in the
// Fortran's operation order, on 1-based column-major arrays.  Only the test
// suite, the smoke check and the benchmark's CPU-baseline leg use it.
// Parity status: unpinned (no reference tests or fixtures exist, and the
// reference cannot be compiled: no Fortran compiler, MPI or PETSc), apart
// from get_mue, get_De, get_Dt and get_nu, which tests/test_golden_coef.py
// checks against the reference's own Python copies of those fits.
//
// Fortran details kept on purpose:
//  * literals written without a d exponent are REAL(4) in Fortran and are
//    rounded to single precision before promotion (e.g. x0 = 1e-4,
//    eps0 = 8.85418782e-12, the fit coefficients of get_mue);  SP() marks them.
//  * x**n with integer n is a chain of multiplications (powi), x**n. with a
//    real exponent is pow().
//  * unary minus binds looser than * and /:  -a*b*c == -(a*b*c).
//  * Fortran SAVEd locals (ptcl_lib.F90:103-109) are all reassigned before use
//    for 2D grids (ny > 1); 1D grids are rejected.
#include "fs_oracle.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

inline double SP(float f) { return (double)f; }   // REAL(4) literal promoted

// powi chains for integer powers (x**n in Fortran)
inline double p2(double x) { return x * x; }
inline double p3(double x) { return p2(x) * x; }
inline double p4(double x) { double t = p2(x); return t * t; }
inline double p5(double x) { return p3(x) * p2(x); }
inline double p6(double x) { double t = p3(x); return t * t; }
inline double p7(double x) { return p4(x) * p3(x); }
inline double p8(double x) { double t = p4(x); return t * t; }
inline double p9(double x) { return p6(x) * p3(x); }
inline double p10(double x) { double t = p5(x); return t * t; }
inline double p11(double x) { return p6(x) * p5(x); }

std::string g_create_error;

// ---------------------------------------------------------------- constants
// props.F90:24-47 and ptcl_props.F90:5-25
struct Consts {
    double pi, eps0, mu0, c0, e, kb, me, x0, ph0, t0, wp02, w2;
    double tg, p, ninf, n_zero;
    double mi, mui, ti, vi, Di, mm, Dm, k_r, k_mp, k_2q, k_3q;
    double h_ir, h_ex, h_si, h_sc, gam;
    double x03;   // x0**3
    double cap;
};

Consts make_consts(const fs_config &c) {
    Consts k;
    k.pi = 4.0 * std::atan(1.0);
    k.eps0 = SP(8.85418782e-12f);
    k.mu0 = 4 * k.pi * SP(1e-7f);
    k.c0 = 1.0 / std::sqrt(k.eps0 * k.mu0);
    k.e = SP(1.60217646e-19f);
    k.kb = SP(1.3806503e-23f);
    k.me = 9.10938188e-31;
    k.x0 = SP(1e-4f);
    k.ph0 = k.e / (k.eps0 * k.x0);
    k.t0 = SP(1e-6f);
    k.x03 = k.x0 * k.x0 * k.x0;
    k.wp02 = (k.t0 * k.t0) * (k.e * k.e) / (k.eps0 * k.x03 * k.me);
    k.w2 = (k.t0 * SP(14e9f)) * (k.t0 * SP(14e9f));
    k.tg = c.tg_k;
    k.p = c.p_torr;
    k.ninf = k.p * 101325.0 / 760.0 / k.kb / k.tg * k.x03;
    k.n_zero = SP(1e8f) * k.x03;
    k.mi = 1.67262178e-27 * 39.948;
    k.mui = 1.45e3 / k.p * 1e-4 * k.ph0 * k.t0 / (k.x0 * k.x0);
    k.ti = k.tg;
    k.vi = std::sqrt((8.0 * k.kb * k.ti) / (k.pi * k.mi)) * k.t0 / k.x0;
    k.Di = k.mui * (k.kb * k.ti / k.e) / k.ph0;
    k.mm = k.mi;
    k.Dm = 2.42e18 * k.x0 / k.ninf / 1e2 * k.t0;
    k.k_r = 2e-7 / 1e6 / k.x03 * k.t0;
    k.k_mp = 6.2e-10 / 1.0e6 / k.x03 * k.t0;
    k.k_2q = 3e-15 / 1e6 / k.x03 * k.t0;
    k.k_3q = 1.1e-31 / 1.0e12 / (k.x03 * k.x03) * k.t0;
    k.h_ir = 15.80 / k.ph0;
    k.h_ex = 11.56 / k.ph0;
    k.h_si = 4.14 / k.ph0;
    k.h_sc = -11.56 / k.ph0;
    k.gam = c.gam;
    k.cap = 1e-11 * k.ph0 / k.e;   // circ_lib.F90:221
    return k;
}

// ------------------------------------------------ coefficient fits (reference)
// ptcl_props.F90:182-429, evaluated at nondimensional mean energy T.
struct Fits {
    const Consts &k;
    explicit Fits(const Consts &kk) : k(kk) {}

    double beta(double T) const {                        // :182-192
        const double a = 11.604505e3;
        double x = std::log10(std::min(T * k.ph0 / 1.5 * a, 5e4));
        return std::pow(10.0, 0.944 - 0.665 * (x - SP(2.48f))) * 1e-13 * k.t0 / k.x03;
    }
    double mue(double T) const {                         // :194-221
        double x = std::log(std::max(2.34e-1, std::min(1.57e2, T * k.ph0)));
        double s;
        if (x < SP(std::log(5.119f)))
            s = SP(58.1133016145f) + SP(-0.984082217962f) * x + SP(-0.164770900119f) * p2(x)
              + SP(-0.142058042584f) * p3(x) + SP(-0.0637079234081f) * p4(x)
              + SP(0.0436642742558f) * p5(x);
        else
            s = SP(70.7846754548f) + SP(-22.7558138237f) * x + SP(12.8366493242f) * p2(x)
              + SP(-3.57242763244f) * p3(x) + SP(0.486276623664f) * p4(x)
              + SP(-0.0259045697422f) * p5(x);
        return std::exp(s) * k.x0 / k.ninf * k.t0 * k.ph0;
    }
    double mut(double T) const {                         // :223-250
        double x = std::log(std::max(2.34e-1, std::min(1.57e2, T * k.ph0)));
        double s;
        if (x < SP(std::log(5.119f)))
            s = SP(58.1354622038f) + SP(-1.29918391109f) * x + SP(-0.106559658509f) * p2(x)
              + SP(-0.0202265418394f) * p3(x) + SP(-0.0286667333915f) * p4(x)
              + SP(0.022457210094f) * p5(x);
        else
            s = SP(68.2627663433f) + SP(-19.3524000831f) * x + SP(11.3251980583f) * p2(x)
              + SP(-3.24070386509f) * p3(x) + SP(0.449848156054f) * p4(x)
              + SP(-0.0242585762405f) * p5(x);
        return std::exp(s) * k.x0 / k.ninf * k.t0 * k.ph0;
    }
    double De(double T) const {                          // :268-291
        double x = std::log(std::max(2.34e-1, std::min(1.57e2, T * k.ph0)));
        double s = SP(57.7067018813f) + SP(-0.0699892875381f) * x + SP(-0.117645585949f) * p2(x)
                 + SP(0.105390295278f) * p3(x) + SP(-0.102862612604f) * p4(x)
                 + SP(-0.0469171521686f) * p5(x) + SP(0.0584908312121f) * p6(x)
                 + SP(0.000578601715687f) * p7(x) + SP(-0.0122860884883f) * p8(x)
                 + SP(0.00426793748856f) * p9(x) + SP(-0.000590000082557f) * p10(x)
                 + SP(3.00706533201e-05f) * p11(x);
        return std::exp(s) * k.x0 / k.ninf * k.t0;
    }
    double Dt(double T) const {                          // :293-316
        double x = std::log(std::max(2.34e-1, std::min(1.57e2, T * k.ph0)));
        double s = SP(57.7214952841f) + SP(-0.353731464348f) * x + SP(-0.00505156731795f) * p2(x)
                 + SP(0.161173720584f) * p3(x) + SP(-0.196610345869f) * p4(x)
                 + SP(-0.0719115643218f) * p5(x) + SP(0.11874085868f) * p6(x)
                 + SP(-0.00669712724784f) * p7(x) + SP(-0.0236445308504f) * p8(x)
                 + SP(0.00917326671764f) * p9(x) + SP(-0.00135453096483f) * p10(x)
                 + SP(7.26379684461e-05f) * p11(x);
        return std::exp(s) * k.x0 / k.ninf * k.t0;
    }
    double k_ex(double T) const {                        // :318-345
        double x = std::log(std::max(9.611e-1, std::min(1.57e2, T * k.ph0)));
        double s;
        if (x < SP(std::log(5.667f)))
            s = SP(-54.4513453969f) + SP(17.1472529739f) * x + SP(-1.05188982824f) * p2(x)
              + SP(-10.5053010711f) * p3(x) + SP(7.51502551486f) * p4(x)
              + SP(-1.44763942525f) * p5(x);
        else
            s = SP(-150.266369415f) + SP(158.67012941f) * x + SP(-85.5163470769f) * p2(x)
              + SP(23.0655081891f) * p3(x) + SP(-3.0908688844f) * p4(x)
              + SP(0.16403226902f) * p5(x);
        return std::exp(s) * k.t0 / k.x03;
    }
    double k_ir(double T) const {                        // :347-374
        double x = std::log(std::max(1.37, std::min(1.57e2, T * k.ph0)));
        double s;
        if (x < SP(std::log(7.5f)))
            s = SP(-73.27080258f) + SP(-30.1312514721f) * x + SP(138.743842326f) * p2(x)
              + SP(-161.378167125f) * p3(x) + SP(81.9325486193f) * p4(x)
              + SP(-14.9080865672f) * p5(x);
        else
            s = SP(-168.925304837f) + SP(177.113452524f) * x + SP(-92.3047166553f) * p2(x)
              + SP(24.1814225482f) * p3(x) + SP(-3.15463258104f) * p4(x)
              + SP(0.16331188192f) * p5(x);
        return std::exp(s) * k.t0 / k.x03;
    }
    double nu(double T) const {                          // :376-395
        double x = std::log(std::max(2.34e-1, std::min(1.57e2, T * k.ph0)));
        double s = SP(-32.275912575f) + SP(1.45173283977f) * x
                 + SP(0.00936933121094f) * std::pow(x, 2.0) + SP(0.129397015353f) * std::pow(x, 3.0)
                 + SP(-0.0414865809044f) * std::pow(x, 4.0) + SP(-0.0582934303409f) * std::pow(x, 5.0)
                 + SP(0.0309832277826f) * std::pow(x, 6.0) + SP(-0.00542014733763f) * p7(x)
                 + SP(0.000325615321708f) * std::pow(x, 8.0);
        return std::exp(s) / k.x03 * k.ninf * k.t0;
    }
    double k_sc(double T) const {                        // :397-413
        double x = std::log(std::min(16.0, std::max(5e-1, T * k.ph0)));
        double s = SP(-21.4827864151f) + SP(0.457356923276f) * x
                 + SP(-0.555439231606f) * std::pow(x, 2.0) + SP(1.27257798891f) * std::pow(x, 3.0)
                 + SP(-0.67840685073f) * std::pow(x, 4.0) + SP(0.10591014464f) * std::pow(x, 5.0);
        return std::exp(s) / 1.0e6 / k.x03 * k.t0;
    }
    double k_si(double T) const {                        // :415-429
        double x = std::log(std::min(16.0, std::max(5e-1, T * k.ph0)));
        double s = SP(-43.1347385848f) + SP(43.9905424566f) * x
                 + SP(-28.1169537586f) * std::pow(x, 2.0) + SP(8.28853856817f) * std::pow(x, 3.0)
                 + SP(-0.931626144207f) * std::pow(x, 4.0);
        return std::exp(s) / 1.0e6 / k.x03 * k.t0;
    }
    double by_index(int which, double T) const {
        switch (which) {
            case 0: return mue(T);
            case 1: return De(T);
            case 2: return k_ir(T);
            case 3: return k_ex(T);
            case 4: return nu(T);
            case 5: return beta(T);
            case 6: return k_sc(T);
            case 7: return k_si(T);
        }
        return NAN;
    }
};

// Table mode: table_n points log-spaced in mean energy eps [eV] from emin to
// emax; row r holds coefficient r at eps_k = exp(ln emin + k*h), T = eps_k/ph0.
// k_ir is the Arrhenius form A*exp(-Ea/eps) [m^3/s] made nondimensional like
// get_k_ir (ptcl_props.F90:368).  Query: u = (ln(T*ph0) - ln emin) * (n-1)/(ln emax - ln emin)
// clamped to [0, n-1];  value = f_k + (u-k)*(f_{k+1}-f_k),  k = min(floor(u), n-2).
struct Table {
    int n = 0;
    double lemin = 0, lemax = 0, inv_h = 0;
    std::vector<double> v;   // 8 rows x n

    void build(const fs_config &c, const Consts &k) {
        Fits f(k);
        n = c.table_n;
        lemin = std::log(c.table_emin_ev);
        lemax = std::log(c.table_emax_ev);
        double h = (lemax - lemin) / (double)(n - 1);
        inv_h = (double)(n - 1) / (lemax - lemin);
        v.assign((size_t)8 * n, 0.0);
        for (int i = 0; i < n; i++) {
            double eps = std::exp(lemin + (double)i * h);
            double T = eps / k.ph0;
            for (int r = 0; r < 8; r++) v[(size_t)r * n + i] = f.by_index(r, T);
            v[(size_t)2 * n + i] = c.kir_arrh_a * std::exp(-c.kir_arrh_e / eps) * k.t0 / k.x03;
        }
    }
    double interp(int row, double T, double ph0) const {
        double x = std::log(T * ph0);
        double u = (x - lemin) * inv_h;
        if (!(u >= 0.0)) u = 0.0;
        if (u > (double)(n - 1)) u = (double)(n - 1);
        int i = (int)u;
        if (i > n - 2) i = n - 2;
        double w = u - (double)i;
        const double *t = &v[(size_t)row * n];
        return t[i] + w * (t[i + 1] - t[i]);
    }
};

// ---------------------------------------------------------------- arrays
struct F2 {                          // real(8) a(ld, nj)   (1-based)
    std::vector<double> a;
    int ld = 0, nj = 0;
    void init(int l, int j, double v = 0) { ld = l; nj = j; a.assign((size_t)l * j, v); }
    double &operator()(int i, int j) { return a[(size_t)(i - 1) + (size_t)(j - 1) * ld]; }
    double operator()(int i, int j) const { return a[(size_t)(i - 1) + (size_t)(j - 1) * ld]; }
};
struct F3 {                          // real(8) a(ld, nj, nl)
    std::vector<double> a;
    int ld = 0, nj = 0, nl = 0;
    void init(int l, int j, int k, double v = 0) { ld = l; nj = j; nl = k; a.assign((size_t)l * j * k, v); }
    double &operator()(int i, int j, int l) { return a[(size_t)(i - 1) + ((size_t)(j - 1) + (size_t)(l - 1) * nj) * ld]; }
    double operator()(int i, int j, int l) const { return a[(size_t)(i - 1) + ((size_t)(j - 1) + (size_t)(l - 1) * nj) * ld]; }
    double *lev(int l) { return &a[(size_t)(l - 1) * nj * ld]; }
    void copy_level(int dst, int src) {
        std::memcpy(lev(dst), lev(src), sizeof(double) * (size_t)nj * ld);
    }
};

}  // namespace

// ------------------------------------------------------------------- context
struct or_ctx {
    fs_config cfg;
    Consts k;
    Table tab;
    int bx, by, nx, ny;
    int solver;
    std::vector<double> dx, dlx, dy, dly, r;     // 1-based storage (index 0 unused)
    std::vector<int> tx, ty;                      // type_x/type_y (1..bx,1..by)
    double t = 0, dt = 0;
    // module state
    F3 ni, ne, nt, nm, ki, ke, kt, km;
    F2 ph, ph_mi;
    double err_prev = 1.0, t_m = 1e9;
    double Vmax, Vsrc, Vd_pl, Vd_mi, Vd_or, Ida = 0, Idc = 0;
    double kv[6] = {0, 0, 0, 0, 0, 0};   // circ_lib.F90:8, kv(1..5)
    // sfc_lib module state (sfc_lib.F90:7): surface charge of the dielectric
    // wall per column, 1-based (1..bx+2), and its Merson stage slopes
    std::vector<double> sig_pl, sig_mi, sig_or, ks;   // ks(i, stage) at i + (stage - 1) * (bx + 3)
    bool rwall = false;                                // some node has type_y == 3
    double err_cur = 0;
    double dt_step = 0;
    long ts = 0;
    fs_stats st;
    std::string err;

    int type_x(int i, int j) const { return tx[(size_t)(i - 1) + (size_t)(j - 1) * bx]; }
    int type_y(int i, int j) const { return ty[(size_t)(i - 1) + (size_t)(j - 1) * bx]; }
    double DX(int i) const { return dx[i]; }
    double DLX(int i) const { return dlx[i]; }
    double DY(int j) const { return dy[j]; }
    double DLY(int j) const { return dly[j]; }
    double R(int j) const { return r[j]; }

    // coefficient access through the configured mode
    double coef(int which, double T) const {
        if (cfg.coef_mode == FS_COEF_TABLE) return tab.interp(which, T, k.ph0);
        Fits f(k);
        return f.by_index(which, T);
    }
    double get_mue(double T) const { return coef(0, T); }
    double get_De(double T) const { return coef(1, T); }
    double get_k_ir(double T) const { return coef(2, T); }
    double get_k_ex(double T) const { return coef(3, T); }
    double get_nu(double T) const { return coef(4, T); }
    double get_beta(double T) const { return coef(5, T); }
    double get_k_sc(double T) const { return coef(6, T); }
    double get_k_si(double T) const { return coef(7, T); }
    double get_mut(double T) const { Fits f(k); return f.mut(T); }
    double get_Dt(double T) const { Fits f(k); return f.Dt(T); }
};

namespace {

// flags raised inside cell loops (get_Te negative density, NaN checks)
struct Flags { int neg = 0, nan = 0, bnan = 0; };

// get_Flux, ptcl_props.F90:142-165
inline double get_flux(double E, double dh, int q, double mu, double D, double nl, double nr) {
    const double tol = SP(1e-12f);
    double v = (double)q * mu * E;
    double arg = v * dh / D;
    double flux;
    if (std::fabs((double)q * E) < tol) {
        flux = D * (nl - nr) / dh;
    } else if (std::fabs(arg) < 1e-2) {
        // Same function in its Bernoulli form, (D/dh)(B(-a) nl - B(a) nr) with
        // B(x) = x/(e^x - 1) = 1 - x/2 + x^2/12 - x^4/720 + O(x^6).  The closed
        // form below divides by 1 - exp(-a), which carries a relative error
        // ~1e-16/|a| and is exactly 0 for |a| < 1.1e-16 (a division by zero the
        // reference hits where E is rounding noise just above the 1e-12 cut).
        double a2 = arg * arg;
        flux = D * ((nl - nr) + 0.5 * arg * (nl + nr) + a2 * (1.0 / 12.0 - a2 / 720.0) * (nl - nr)) / dh;
    } else if (arg > 0) {
        flux = v * (nl - nr * std::exp(std::max(-arg, -100.0))) / (1.0 - std::exp(std::max(-arg, -100.0)));
    } else {
        flux = v * (nr - nl * std::exp(std::max(arg, -100.0))) / (1.0 - std::exp(std::max(arg, -100.0)));
    }
    return flux;
}

// get_Te, ptcl_props.F90:167-180 (the Fortran stops; here a flag is raised)
inline double get_Te(double nte, double ne, Flags &fl) {
    if ((nte >= 0.0) && (ne >= 0.0)) return nte / ne;
    fl.neg = 1;
    return 1e-8;
}

// dFdPh, lapl_lib.F90:611-636
inline double dfdph(double E_pl, double E_mi, int q, double mu, double D, double dx,
                    double n1, double n2, Flags *fl) {
    const double tol = 1e-12;
    double v_mi = (double)q * mu * E_mi;
    double v_pl = (double)q * mu * E_pl;
    double a_mi = v_mi * dx / D;
    (void)v_pl;
    double df;
    if (std::fabs(v_mi) < tol) {
        df = 0.0;
    } else if (std::fabs(a_mi) < 0.05) {
        // Same function as below, evaluated by its series: with the SG flux
        // F = (D/dx)(B(-a) n1 - B(a) n2), B(x) = x/(e^x - 1), dF/dv =
        // (n1+n2)/2 + (n1-n2)(a/6 - a^3/180 + a^5/5040) + O(a^7).  The closed
        // form cancels here (two terms ~ (n1-n2)/a leave ~(n1+n2)/2 with an
        // error ~2e-16 |n1-n2| / a^2, all digits lost for |a| < 1e-8), so the
        // reference's own value is rounding noise near a = 0.
        double dn = n1 - n2, a2 = a_mi * a_mi;
        df = 0.5 * (n1 + n2) + dn * a_mi * (1.0 / 6.0 - a2 * (1.0 / 180.0 - a2 / 5040.0));
    } else if (a_mi > 0) {
        double ex = std::exp(-a_mi);
        df = (n1 - n2 * ex) / (1.0 - ex) + v_mi * ex * (n2 - n1) / ((1.0 - ex) * (1.0 - ex)) * dx / D;
    } else {
        double ex = std::exp(a_mi);
        df = (n2 - n1 * ex) / (1.0 - ex) + v_mi * ex * (n2 - n1) / ((1.0 - ex) * (1.0 - ex)) * dx / D;
    }
    if (std::isnan(df) && fl) fl->nan = 1;
    return df;
}

// ptclEqn, ptcl_lib.F90:99-550 (Em = 0, ny > 1)
void ptclEqn(or_ctx &c, int i, int j, int stage, Flags &fl, double &t_m_loc) {
    const Consts &k = c.k;
    const F2 &ph = c.ph;
    const bool four = c.cfg.nspecies == 4;
    auto NI = [&](int a, int b) { return c.ni(a, b, 2); };
    auto NE = [&](int a, int b) { return c.ne(a, b, 2); };
    auto NT = [&](int a, int b) { return c.nt(a, b, 2); };
    auto NM = [&](int a, int b) { return four ? c.nm(a, b, 2) : 0.0; };
    const double f53 = 5.0 / 3.0;
    double a, Ex[2], Ey[2], Te[3] = {0, 0, 0}, mue[2] = {0, 0}, mut[2] = {0, 0}, De[2] = {0, 0}, Dt[2] = {0, 0};
    double fluxi_x[2] = {0, 0}, fluxi_y[2] = {0, 0}, fluxe_x[2] = {0, 0}, fluxe_y[2] = {0, 0};
    double fluxt_x[2] = {0, 0}, fluxt_y[2] = {0, 0}, fluxm_x[2] = {0, 0}, fluxm_y[2] = {0, 0};
    double ve;
    const int tx = c.type_x(i - 1, j - 1), ty = c.type_y(i - 1, j - 1);

    // X-dir fields (:112-121)
    if (tx == -1) {
        Ex[0] = 0.0;
        Ex[1] = -(ph(i + 1, j) - ph(i, j)) / c.DX(i);
    } else if (tx == 1) {
        Ex[0] = -(ph(i, j) - ph(i - 1, j)) / c.DX(i - 1);
        Ex[1] = 0.0;
    } else {
        Ex[0] = -(ph(i, j) - ph(i - 1, j)) / c.DX(i - 1);
        Ex[1] = -(ph(i + 1, j) - ph(i, j)) / c.DX(i);
    }

    // X-dir fluxes (:123-282)
    if (tx == 0) {
        Te[0] = get_Te(NT(i - 1, j), NE(i - 1, j), fl);
        Te[1] = get_Te(NT(i, j), NE(i, j), fl);
        Te[2] = get_Te(NT(i + 1, j), NE(i + 1, j), fl);
        mue[0] = 5e-1 * (c.get_mue(Te[0]) + c.get_mue(Te[1]));
        mue[1] = 5e-1 * (c.get_mue(Te[1]) + c.get_mue(Te[2]));
        De[0] = 5e-1 * (c.get_De(Te[0]) + c.get_De(Te[1]));
        De[1] = 5e-1 * (c.get_De(Te[1]) + c.get_De(Te[2]));
        mut[0] = f53 * mue[0]; mut[1] = f53 * mue[1];
        Dt[0] = f53 * De[0]; Dt[1] = f53 * De[1];
        fluxi_x[0] = get_flux(Ex[0], c.DX(i - 1), 1, k.mui, k.Di, NI(i - 1, j), NI(i, j));
        fluxe_x[0] = get_flux(Ex[0], c.DX(i - 1), -1, mue[0], De[0], NE(i - 1, j), NE(i, j));
        fluxt_x[0] = get_flux(Ex[0], c.DX(i - 1), -1, mut[0], Dt[0], NT(i - 1, j), NT(i, j));
        fluxm_x[0] = -k.Dm * (NM(i, j) - NM(i - 1, j)) / c.DX(i - 1);
        fluxi_x[1] = get_flux(Ex[1], c.DX(i), 1, k.mui, k.Di, NI(i, j), NI(i + 1, j));
        fluxe_x[1] = get_flux(Ex[1], c.DX(i), -1, mue[1], De[1], NE(i, j), NE(i + 1, j));
        fluxt_x[1] = get_flux(Ex[1], c.DX(i), -1, mut[1], Dt[1], NT(i, j), NT(i + 1, j));
        fluxm_x[1] = -k.Dm * (NM(i + 1, j) - NM(i, j)) / c.DX(i);
    } else if (tx < 0) {
        Te[1] = get_Te(NT(i, j), NE(i, j), fl);
        Te[2] = get_Te(NT(i + 1, j), NE(i + 1, j), fl);
        mue[1] = 5e-1 * (c.get_mue(Te[1]) + c.get_mue(Te[2]));
        De[1] = 5e-1 * (c.get_De(Te[1]) + c.get_De(Te[2]));
        mut[0] = f53 * mue[0]; mut[1] = f53 * mue[1];
        Dt[0] = f53 * De[0]; Dt[1] = f53 * De[1];
        fluxi_x[1] = get_flux(Ex[1], c.DX(i), 1, k.mui, k.Di, NI(i, j), NI(i + 1, j));
        fluxe_x[1] = get_flux(Ex[1], c.DX(i), -1, mue[1], De[1], NE(i, j), NE(i + 1, j));
        fluxt_x[1] = get_flux(Ex[1], c.DX(i), -1, mut[1], Dt[1], NT(i, j), NT(i + 1, j));
        fluxm_x[1] = -k.Dm * (NM(i + 1, j) - NM(i, j)) / c.DX(i);
        if (tx == -2) {
            a = (ph(i - 1, j) > ph(i, j)) ? 1.0 : 0.0;
            mue[0] = c.get_mue(Te[1]);
            mut[0] = f53 * mue[0]; mut[1] = f53 * mue[1];
            ve = std::sqrt((16.0 * k.e * k.ph0 * Te[1]) / (3.0 * k.pi * k.me)) * k.t0 / k.x0;
            fluxi_x[0] = (1.0 - a) * k.mui * Ex[0] * NI(i, j) - 2.5e-1 * k.vi * NI(i, j);
            fluxe_x[0] = -(a * mue[0] * Ex[0] * NE(i, j)) - 2.5e-1 * ve * NE(i, j) - k.gam * fluxi_x[0];
            fluxt_x[0] = -(a * mut[0] * Ex[0] * NT(i, j)) - 1.0 / 3.0 * ve * NT(i, j) - k.gam * Te[1] * fluxi_x[0];
            fluxm_x[0] = -(5e-1 * k.vi * NM(i, j));
        } else if (tx == -1) {
            fluxi_x[0] = 0.0; fluxe_x[0] = 0.0; fluxt_x[0] = 0.0; fluxm_x[0] = 0.0;
        }
    } else if (tx > 0) {
        Te[0] = get_Te(NT(i - 1, j), NE(i - 1, j), fl);
        Te[1] = get_Te(NT(i, j), NE(i, j), fl);
        mue[0] = 5e-1 * (c.get_mue(Te[0]) + c.get_mue(Te[1]));
        De[0] = 5e-1 * (c.get_De(Te[0]) + c.get_De(Te[1]));
        mut[0] = f53 * mue[0]; mut[1] = f53 * mue[1];
        Dt[0] = f53 * De[0]; Dt[1] = f53 * De[1];
        fluxi_x[0] = get_flux(Ex[0], c.DX(i - 1), 1, k.mui, k.Di, NI(i - 1, j), NI(i, j));
        fluxe_x[0] = get_flux(Ex[0], c.DX(i - 1), -1, mue[0], De[0], NE(i - 1, j), NE(i, j));
        fluxt_x[0] = get_flux(Ex[0], c.DX(i - 1), -1, mut[0], Dt[0], NT(i - 1, j), NT(i, j));
        fluxm_x[0] = -k.Dm * (NM(i, j) - NM(i - 1, j)) / c.DX(i - 1);
        if (tx == 2) {
            a = (ph(i + 1, j) > ph(i, j)) ? 1.0 : 0.0;
            mue[1] = c.get_mue(Te[1]);
            mut[0] = f53 * mue[0]; mut[1] = f53 * mue[1];
            ve = std::sqrt((16.0 * k.e * k.ph0 * Te[1]) / (3.0 * k.pi * k.me)) * k.t0 / k.x0;
            fluxi_x[1] = (1.0 - a) * k.mui * Ex[1] * NI(i, j) + 2.5e-1 * k.vi * NI(i, j);
            fluxe_x[1] = -(a * mue[1] * Ex[1] * NE(i, j)) + 2.5e-1 * ve * NE(i, j) - k.gam * fluxi_x[1];
            fluxt_x[1] = -(a * mut[1] * Ex[1] * NT(i, j)) + 1.0 / 3.0 * ve * NT(i, j) - k.gam * Te[1] * fluxi_x[1];
            fluxm_x[1] = 5e-1 * k.vi * NM(i, j);
        } else if (tx == 1) {
            fluxi_x[1] = 0.0; fluxe_x[1] = 0.0; fluxt_x[1] = 0.0; fluxm_x[1] = 0.0;
        }
    }

    // Y-dir fields and fluxes (:284-443)
    if (ty == -1) {
        Ey[0] = 0.0;
        Ey[1] = -(ph(i, j + 1) - ph(i, j)) / c.DY(j);
    } else if (ty == 1) {
        Ey[0] = -(ph(i, j) - ph(i, j - 1)) / c.DY(j - 1);
        Ey[1] = 0.0;
    } else if (ty == 3) {
        Ey[0] = -(ph(i, j) - ph(i, j - 1)) / c.DY(j - 1);
        Ey[1] = -c.sig_mi[i];   // dielectric surface charge (:292-294)
    } else {
        Ey[0] = -(ph(i, j) - ph(i, j - 1)) / c.DY(j - 1);
        Ey[1] = -(ph(i, j + 1) - ph(i, j)) / c.DY(j);
    }
    if (ty == 0) {
        Te[0] = get_Te(NT(i, j - 1), NE(i, j - 1), fl);
        Te[1] = get_Te(NT(i, j), NE(i, j), fl);
        Te[2] = get_Te(NT(i, j + 1), NE(i, j + 1), fl);
        mue[0] = 5e-1 * (c.get_mue(Te[0]) + c.get_mue(Te[1]));
        mue[1] = 5e-1 * (c.get_mue(Te[1]) + c.get_mue(Te[2]));
        De[0] = 5e-1 * (c.get_De(Te[0]) + c.get_De(Te[1]));
        De[1] = 5e-1 * (c.get_De(Te[1]) + c.get_De(Te[2]));
        mut[0] = f53 * mue[0]; mut[1] = f53 * mue[1];
        Dt[0] = f53 * De[0]; Dt[1] = f53 * De[1];
        fluxi_y[0] = get_flux(Ey[0], c.DY(j - 1), 1, k.mui, k.Di, NI(i, j - 1), NI(i, j));
        fluxe_y[0] = get_flux(Ey[0], c.DY(j - 1), -1, mue[0], De[0], NE(i, j - 1), NE(i, j));
        fluxt_y[0] = get_flux(Ey[0], c.DY(j - 1), -1, mut[0], Dt[0], NT(i, j - 1), NT(i, j));
        fluxm_y[0] = -k.Dm * (NM(i, j) - NM(i, j - 1)) / c.DY(j - 1);
        fluxi_y[1] = get_flux(Ey[1], c.DY(j), 1, k.mui, k.Di, NI(i, j), NI(i, j + 1));
        fluxe_y[1] = get_flux(Ey[1], c.DY(j), -1, mue[1], De[1], NE(i, j), NE(i, j + 1));
        fluxt_y[1] = get_flux(Ey[1], c.DY(j), -1, mut[1], Dt[1], NT(i, j), NT(i, j + 1));
        fluxm_y[1] = -k.Dm * (NM(i, j + 1) - NM(i, j)) / c.DY(j);
    } else if (ty < 0) {
        Te[1] = get_Te(NT(i, j), NE(i, j), fl);
        Te[2] = get_Te(NT(i, j + 1), NE(i, j + 1), fl);
        mue[1] = 5e-1 * (c.get_mue(Te[1]) + c.get_mue(Te[2]));
        De[1] = 5e-1 * (c.get_De(Te[1]) + c.get_De(Te[2]));
        mut[0] = f53 * mue[0]; mut[1] = f53 * mue[1];
        Dt[0] = f53 * De[0]; Dt[1] = f53 * De[1];
        fluxi_y[1] = get_flux(Ey[1], c.DY(j), 1, k.mui, k.Di, NI(i, j), NI(i, j + 1));
        fluxe_y[1] = get_flux(Ey[1], c.DY(j), -1, mue[1], De[1], NE(i, j), NE(i, j + 1));
        fluxt_y[1] = get_flux(Ey[1], c.DY(j), -1, mut[1], Dt[1], NT(i, j), NT(i, j + 1));
        fluxm_y[1] = -k.Dm * (NM(i, j + 1) - NM(i, j)) / c.DY(j);
        fluxi_y[0] = 0.0; fluxe_y[0] = 0.0; fluxt_y[0] = 0.0; fluxm_y[0] = 0.0;
    } else if (ty > 0) {
        Te[0] = get_Te(NT(i, j - 1), NE(i, j - 1), fl);
        Te[1] = get_Te(NT(i, j), NE(i, j), fl);
        mue[0] = 5e-1 * (c.get_mue(Te[0]) + c.get_mue(Te[1]));
        De[0] = 5e-1 * (c.get_De(Te[0]) + c.get_De(Te[1]));
        mut[0] = f53 * mue[0]; mut[1] = f53 * mue[1];
        Dt[0] = f53 * De[0]; Dt[1] = f53 * De[1];
        fluxi_y[0] = get_flux(Ey[0], c.DY(j - 1), 1, k.mui, k.Di, NI(i, j - 1), NI(i, j));
        fluxe_y[0] = get_flux(Ey[0], c.DY(j - 1), -1, mue[0], De[0], NE(i, j - 1), NE(i, j));
        fluxt_y[0] = get_flux(Ey[0], c.DY(j - 1), -1, mut[0], Dt[0], NT(i, j - 1), NT(i, j));
        fluxm_y[0] = -k.Dm * (NM(i, j) - NM(i, j - 1)) / c.DY(j - 1);
        if (ty == 3) {
            Te[1] = get_Te(NT(i, j), NE(i, j), fl);
            mue[1] = c.get_mue(Te[1]);
            De[1] = c.get_De(Te[1]);
            mut[1] = c.get_mut(Te[1]);
            Dt[1] = c.get_Dt(Te[1]);
            fluxi_y[1] = get_flux(Ey[1], c.DY(j), 1, k.mui, k.Di, NI(i, j), 0.0);
            fluxe_y[1] = get_flux(Ey[1], c.DY(j), -1, mue[1], De[1], NE(i, j), 0.0);
            fluxt_y[1] = get_flux(Ey[1], c.DY(j), -1, mut[1], Dt[1], NT(i, j), 0.0);
            fluxm_y[1] = k.Dm * NM(i, j) / c.DY(j);
        } else if (ty == 2) {
            a = (ph(i, j + 1) > ph(i, j)) ? 1.0 : 0.0;
            mue[1] = c.get_mue(Te[1]);
            mut[0] = f53 * mue[0]; mut[1] = f53 * mue[1];
            ve = std::sqrt((16.0 * k.e * k.ph0 * Te[1]) / (3.0 * k.pi * k.me)) * k.t0 / k.x0;
            fluxi_y[1] = (1.0 - a) * k.mui * Ey[1] * NI(i, j) + 2.5e-1 * k.vi * NI(i, j);
            // the reference uses the x-direction ion flux here (ptcl_lib.F90:429,433)
            fluxe_y[1] = -(a * mue[1] * Ey[1] * NE(i, j)) + 2.5e-1 * ve * NE(i, j) - k.gam * fluxi_x[1];
            fluxt_y[1] = -(a * mut[1] * Ey[1] * NT(i, j)) + 1.0 / 3.0 * ve * NT(i, j) - k.gam * Te[1] * fluxi_x[1];
            fluxm_y[1] = 5e-1 * k.vi * NM(i, j);
        } else {
            fluxi_y[1] = 0.0; fluxe_y[1] = 0.0; fluxt_y[1] = 0.0; fluxm_y[1] = 0.0;
        }
    }

    // flux gradients (:445-480)
    double dfi_dx = (fluxi_x[1] - fluxi_x[0]) / c.DLX(i - 1);
    double dfe_dx = (fluxe_x[1] - fluxe_x[0]) / c.DLX(i - 1);
    double dft_dx = (fluxt_x[1] - fluxt_x[0]) / c.DLX(i - 1);
    double dfm_dx = (fluxm_x[1] - fluxm_x[0]) / c.DLX(i - 1);
    fluxe_x[0] = (fluxe_x[1] + fluxe_x[0]) / 2.0;
    Ex[0] = (Ex[0] + Ex[1]) / 2.0;
    double dfi_dy, dfe_dy, dft_dy, dfm_dy;
    if (c.cfg.cyl) {
        double rp = (c.R(j + 1) + c.R(j)), rm = (c.R(j) + c.R(j - 1));
        dfi_dy = (fluxi_y[1] * rp / 2.0 - fluxi_y[0] * rm / 2.0) / c.DLY(j - 1) / c.R(j);
        dfe_dy = (fluxe_y[1] * rp / 2.0 - fluxe_y[0] * rm / 2.0) / c.DLY(j - 1) / c.R(j);
        dft_dy = (fluxt_y[1] * rp / 2.0 - fluxt_y[0] * rm / 2.0) / c.DLY(j - 1) / c.R(j);
        dfm_dy = (fluxm_y[1] * rp / 2.0 - fluxm_y[0] * rm / 2.0) / c.DLY(j - 1) / c.R(j);
    } else {
        dfi_dy = (fluxi_y[1] - fluxi_y[0]) / c.DLY(j - 1);
        dfe_dy = (fluxe_y[1] - fluxe_y[0]) / c.DLY(j - 1);
        dft_dy = (fluxt_y[1] - fluxt_y[0]) / c.DLY(j - 1);
        dfm_dy = (fluxm_y[1] - fluxm_y[0]) / c.DLY(j - 1);
    }
    fluxe_y[0] = (fluxe_y[1] + fluxe_y[0]) / 2.0;
    Ey[0] = (Ey[0] + Ey[1]) / 2.0;

    // sources (:482-524)
    double T2 = Te[1];
    double k_ir = c.get_k_ir(T2), k_sc = c.get_k_sc(T2), k_si = c.get_k_si(T2);
    double k_ex = c.get_k_ex(T2), nu = c.get_nu(T2), beta = c.get_beta(T2);
    double ne_ = NE(i, j), ni_ = NI(i, j), nm_ = NM(i, j);
    double term_sie = k_ir * k.ninf * ne_ - beta * ni_ * ne_ + k_si * nm_ * ne_ + k.k_mp * p2(nm_);
    double term_sm = k_ex * k.ninf * ne_ - k_si * nm_ * ne_ - k_sc * nm_ * ne_ - k.k_r * nm_ * ne_
                   - 2.0 * k.k_mp * p2(nm_) - k.k_2q * k.ninf * nm_ - k.k_3q * p2(k.ninf) * nm_;
    double term_st1 = -(fluxe_x[0] * Ex[0] + fluxe_y[0] * Ey[0]);
    double term_st2 = -(ne_ * nu * k.me / k.mi * (T2 / 1.5 - k.tg * k.kb / k.e / k.ph0));
    const double Em = 0.0;
    double term_st3 = -(k.h_ir * k_ir * k.ninf * ne_) - k.h_si * k_si * nm_ * ne_
                    - k.h_ex * k_ex * k.ninf * ne_ + ne_ * k.wp02 * Em / std::sqrt(k.w2 + p2(nu));
    double vki = -dfi_dx - dfi_dy + term_sie;
    double vke = -dfe_dx - dfe_dy + term_sie;
    double vkt = -dft_dx - dft_dy + term_st1 + term_st2 + term_st3;
    double vkm = -dfm_dx - dfm_dy + term_sm;
    c.ki(i, j, stage) = vki;
    c.ke(i, j, stage) = vke;
    c.kt(i, j, stage) = vkt;
    if (four) c.km(i, j, stage) = vkm;
    if (stage == 5) t_m_loc = std::min(t_m_loc, 1.0 / (mue[1] * ne_ + k.mui * ni_));
    if (std::isnan(vki) || std::isnan(vke) || std::isnan(vkt) || (four && std::isnan(vkm))) fl.nan = 1;
}

// rk_step order 4 (Merson), ptcl_props.F90:71-139.  Returns the stage-5 error
// sum; the whole-array sum of the reference is taken column by column
// (per-j partial sums added in j order) so that the result does not depend on
// the number of threads.
double rk_step(or_ctx &c, F3 &n, F3 &kk, int stage, double dt, double n_min) {
    const int bx = c.bx, by = c.by, ld = bx + 2;
    const double abs_tol = c.cfg.abs_tol, rel_tol = c.cfg.rel_tol;
    if (stage <= 4) {
#pragma omp parallel for schedule(static)
        for (int j = 2; j <= by + 1; j++)
            for (int i = 2; i <= bx + 1; i++) {
                double v;
                if (stage == 1) v = n(i, j, 3) + kk(i, j, 1) * dt / 3.0;
                else if (stage == 2) v = n(i, j, 3) + dt * (kk(i, j, 1) + kk(i, j, 2)) / 6.0;
                else if (stage == 3) v = n(i, j, 3) + dt * (kk(i, j, 1) + kk(i, j, 3) * 3.0) / 8.0;
                else v = n(i, j, 3) + dt * (kk(i, j, 1) - kk(i, j, 3) * 3.0 + kk(i, j, 4) * 4.0) / 2.0;
                n(i, j, 2) = v;
            }
        double *a2 = n.lev(2);
        for (size_t q = 0; q < (size_t)ld * (by + 2); q++) a2[q] = std::max(a2[q], n_min);
        return 0.0;
    }
#pragma omp parallel for schedule(static)
    for (int j = 2; j <= by + 1; j++)
        for (int i = 2; i <= bx + 1; i++)
            n(i, j, 1) = n(i, j, 3) + dt * (kk(i, j, 1) + kk(i, j, 4) * 4.0 + kk(i, j, 5)) / 6.0;
    double *a1 = n.lev(1);
    for (size_t q = 0; q < (size_t)ld * (by + 2); q++) a1[q] = std::max(a1[q], n_min);
    std::vector<double> col(by + 2, 0.0);
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= by + 2; j++) {
        double s = 0.0;
        for (int i = 1; i <= bx + 2; i++) {
            double err = std::fabs(dt * (kk(i, j, 1) * 2.0 / 30.0 - kk(i, j, 3) * 3.0 / 10.0
                                         + kk(i, j, 4) * 4.0 / 15.0 - kk(i, j, 5) / 30.0));
            double q = err / (abs_tol + rel_tol * std::fabs(n(i, j, 3)));
            s += q * q;
        }
        col[j - 1] = s;
    }
    double tot = 0.0;
    for (int j = 0; j < by + 2; j++) tot += col[j];
    return tot;
}

// electrode current at one face column (circ_lib.F90:102-116 / :135-149)
double circ_face(const or_ctx &c, int il, int j, double dh, Flags &fl) {
    const Consts &k = c.k;
    const int st = 2;
    double Ex = -(c.ph(il + 1, j) - c.ph(il, j)) / dh;
    double Te1 = get_Te(c.nt(il, j, st), c.ne(il, j, st), fl);
    double Te2 = get_Te(c.nt(il + 1, j, st), c.ne(il + 1, j, st), fl);
    double mue = 5e-1 * (c.get_mue(Te1) + c.get_mue(Te2));
    double De = 5e-1 * (c.get_De(Te1) + c.get_De(Te2));
    double flxi = get_flux(Ex, dh, 1, k.mui, k.Di, c.ni(il, j, st), c.ni(il + 1, j, st));
    double flxe = get_flux(Ex, dh, -1, mue, De, c.ne(il, j, st), c.ne(il + 1, j, st));
    return flxi - flxe;
}

// source voltage of circ_step (circ_lib.F90:26-50) at time t
double circ_source(const or_ctx &c, double t) {
    const double pi = c.k.pi, V = c.Vmax;
    switch (c.cfg.rf) {
    case 1: return V * std::sin(pi * t);                                    // AC
    case 2: {                                                               // pulse
        if (t < 2.5e-1) { double s = std::sin(4 * pi * t); return V * (s * s * s); }
        return 0.0;
    }
    case 3: {                                                               // measured pulse shape
        if (t < 2.3e-1) { double s = std::sin(4.0 * pi * t); return V * (s * s); }
        if (t < 3.35e-1) return V * (std::sin(3.81 * pi * (t + 5.85e-2)) * 7.19e-1 + 2.81e-1);
        if (t < 8.2e-1) { double s = std::sin(3.81 * pi * (t + 1.2e-1) / 3.5); return V * ((s * s * s) * (-4.38e-1)); }
        return 0.0;
    }
    default: return V;                                                      // DC
    }
}

// circ_step, circ_lib.F90:19-210 (ny > 1)
void circ_step(or_ctx &c, int stage, Flags &fl) {
    const int bx = c.bx, by = c.by;
    c.Vsrc = circ_source(c, c.t);
    double dr;
    int i = 3;
    c.Ida = 0;
    for (int j = 2; j <= by + 1; j++) {
        if (c.type_x(i - 2, j - 1) == -2) {
            dr = c.cfg.cyl ? c.DY(j - 1) * c.R(j - 1) * 2.0 * c.k.pi : c.DY(j - 1) * c.cfg.w;
            if (c.R(j) < c.cfg.ew) dr = 0.0;
            c.Ida = c.Ida + dr * circ_face(c, i - 1, j, c.DX(i - 1), fl);
        }
    }
    i = bx;
    c.Idc = 0;
    for (int j = 2; j <= by + 1; j++) {
        if (c.type_x(i, j - 1) == 2) {
            dr = c.cfg.cyl ? c.DY(j - 1) * c.R(j - 1) * 2.0 * c.k.pi : c.DY(j - 1) * c.cfg.w;
            if (c.R(j) < c.cfg.ew) dr = 0.0;
            c.Idc = c.Idc + dr * circ_face(c, i, j, c.DX(i), fl);
        }
    }
    // RC circuit of the electrode voltage (:156-174); it drives Vd for rf == 1
    // only, the other sources set Vd_pl = Vd_mi = Vsrc (:176-177)
    const double dt = c.dt;
    double *kv = c.kv;
    kv[stage] = -(c.Idc - (c.Vsrc - c.Vd_mi) / c.cfg.res) / c.k.cap;
    if (stage == 1) c.Vd_mi = c.Vd_or + dt * kv[1] / 3.0;
    else if (stage == 2) c.Vd_mi = c.Vd_or + dt * (kv[1] + kv[2]) / 6.0;
    else if (stage == 3) c.Vd_mi = c.Vd_or + dt * (kv[1] + kv[3] * 3.0) / 8.0;
    else if (stage == 4) c.Vd_mi = c.Vd_or + dt * (kv[1] - kv[3] * 3.0 + kv[4] * 4.0) / 2.0;
    else c.Vd_pl = c.Vd_or + dt * (kv[1] + kv[4] * 4.0 + kv[5]) / 6.0;
    if (c.cfg.rf != 1) c.Vd_pl = c.Vsrc;
    if (c.cfg.rf != 1) c.Vd_mi = c.Vsrc;
    i = 2;
    for (int j = 2; j <= by + 1; j++) {
        if (c.R(j) <= c.cfg.ew) {
            if (c.type_x(i - 1, j - 1) == -2) c.ph(i - 1, j) = (stage == 5 ? c.Vd_pl : c.Vd_mi) / 2.0;
            if (c.type_x(bx, j - 1) == 2) c.ph(bx + 2, j) = (stage == 5 ? c.Vd_pl : c.Vd_mi) / (-2.0);
        }
    }
}

// sfc_step, sfc_lib.F90:19-80: Merson stages of the wall charge on the last
// interior row.  Two points where the oracle has to choose:
//  * ptcl_step passes (ni, ne, nt) to the dummy arguments (ne, ni, nt)
//    (ptcl_lib.F90:52 against sfc_lib.F90:19-23), so the routine's "ne" is
//    the ion density and its "ni" the electron density; kept as written;
//  * the routine tests type_y(i-1, by+1), one column past the end of
//    type_y(bx, by), whose value is whatever memory follows the array; the
//    oracle tests the wall row type_y(i-1, by), as ptclEqn does for the same
//    nodes (ptcl_lib.F90:292).
void sfc_step(or_ctx &c, int stage, Flags &fl) {
    const Consts &k = c.k;
    const int j = c.by + 1, ld = c.bx + 3;
    for (int i = 2; i <= c.bx + 1; i++) {
        if (c.type_y(i - 1, j - 1) == 3) {
            const double ne_a = c.ni(i, j, 2), ni_a = c.ne(i, j, 2), nt_a = c.nt(i, j, 2);
            double Te = get_Te(nt_a, ne_a, fl);
            double mue = c.get_mue(Te);
            double De = c.get_De(Te);
            double fluxi = get_flux(-c.sig_mi[i], c.DY(j), 1, k.mui, k.Di, ni_a, 0.0);
            double fluxe = get_flux(-c.sig_mi[i], c.DY(j), -1, mue, De, ne_a, 0.0);
            c.ks[i + (stage - 1) * ld] = fluxi - fluxe;
        }
    }
    auto K = [&](int i, int s) { return c.ks[i + (s - 1) * ld]; };
    const double dt = c.dt;
    for (int i = 2; i <= c.bx + 1; i++) {
        if (c.type_y(i - 1, j - 1) == 3) {
            if (stage == 1) c.sig_mi[i] = c.sig_or[i] + dt * K(i, 1) / 3.0;
            else if (stage == 2) c.sig_mi[i] = c.sig_or[i] + dt * (K(i, 1) + K(i, 2)) / 6.0;
            else if (stage == 3) c.sig_mi[i] = c.sig_or[i] + dt * (K(i, 1) + K(i, 3) * 3.0) / 8.0;
            else if (stage == 4) c.sig_mi[i] = c.sig_or[i] + dt * (K(i, 1) - K(i, 3) * 3.0 + K(i, 4) * 4.0) / 2.0;
            else c.sig_pl[i] = c.sig_or[i] + dt * (K(i, 1) + K(i, 4) * 4.0 + K(i, 5)) / 6.0;
        }
    }
    // the east/west exchange of the ghost entries (:57-70) has no neighbour
    // on a single block: sig(1) and sig(bx+2) keep their values
}

int flags_to_code(or_ctx &c, const Flags &fl) {
    if (fl.neg) { c.err = "negative density in get_Te"; return FS_ERR_NEG_DENSITY; }
    if (fl.nan) { c.err = "NaN in particle right-hand side"; return FS_ERR_NAN; }
    return FS_OK;
}

// ptcl_step, ptcl_lib.F90:32-97
int ptcl_step(or_ctx &c, int &attempts) {
    const int bx = c.bx, by = c.by;
    const bool four = c.cfg.nspecies == 4;
    int stage = 0;
    attempts = 1;
    for (;;) {
        stage = stage + 1;
        if (stage > 5) break;
        Flags fl;
        double tm = c.t_m;
        std::vector<double> tms(by + 2, 1e300);
        std::vector<Flags> fls(by + 2);
#pragma omp parallel for schedule(static)
        for (int j = 2; j <= by + 1; j++) {
            double tl = tm;
            for (int i = 2; i <= bx + 1; i++) ptclEqn(c, i, j, stage, fls[j], tl);
            tms[j] = tl;
        }
        for (int j = 2; j <= by + 1; j++) {
            tm = std::min(tm, tms[j]);
            fl.neg |= fls[j].neg;
            fl.nan |= fls[j].nan;
        }
        c.t_m = tm;
        int rc = flags_to_code(c, fl);
        if (rc) return rc;
        circ_step(c, stage, fl);
        if (c.rwall) sfc_step(c, stage, fl);
        rc = flags_to_code(c, fl);
        if (rc) return rc;
        double e_ni = rk_step(c, c.ni, c.ki, stage, c.dt, c.k.n_zero);
        double e_ne = rk_step(c, c.ne, c.ke, stage, c.dt, c.k.n_zero);
        double e_nt = rk_step(c, c.nt, c.kt, stage, c.dt, c.k.n_zero / c.k.ph0 / 1e2);
        double e_nm = four ? rk_step(c, c.nm, c.km, stage, c.dt, c.k.n_zero) : 0.0;
        if (stage == 5) {
            double err_cur = std::sqrt(e_ni + e_ne + e_nm + e_nt);
            c.err_cur = err_cur;
            c.dt_step = c.dt;
            if (!c.cfg.adaptive) break;
            double scfac = 8e-1 * std::pow(err_cur, -7e-1 / 4.0) * std::pow(c.err_prev, 4e-1 / 4.0);
            scfac = std::min(2.5, std::max(3e-1, scfac));
            c.dt = scfac * c.dt;
            if (c.dt <= c.cfg.dt_min) { c.err = "minimum timestep reached"; return FS_ERR_MIN_DT; }
            if (err_cur <= 1.0) {
                c.err_prev = err_cur;
            } else {
                stage = 0;
                attempts++;
                c.st.rk_rejects++;
                c.ni.copy_level(1, 3); c.ne.copy_level(1, 3); c.nt.copy_level(1, 3);
                c.ni.copy_level(2, 3); c.ne.copy_level(2, 3); c.nt.copy_level(2, 3);
                if (four) { c.nm.copy_level(1, 3); c.nm.copy_level(2, 3); }
                c.Vd_pl = c.Vd_or;
                c.Vd_mi = c.Vd_or;
                c.sig_pl = c.sig_or;
                c.sig_mi = c.sig_or;
            }
        }
    }
    return FS_OK;
}

// ---------------------------------------------------------------- Poisson
// laplEqn, lapl_lib.F90:123-379 on level-1 densities.
double laplEqn(const or_ctx &c, int i, int j, double dt, Flags &fl) {
    const Consts &k = c.k;
    const F2 &ph = c.ph;
    auto NI = [&](int a, int b) { return c.ni(a, b, 1); };
    auto NE = [&](int a, int b) { return c.ne(a, b, 1); };
    auto NT = [&](int a, int b) { return c.nt(a, b, 1); };
    double dfdx = 0, dfdy = 0, dflxe_x = 0, dflxe_y = 0, dflxi_x = 0, dflxi_y = 0;
    double Ex[2], Ey[2], mue[2] = {0, 0}, De[2] = {0, 0}, Te[3] = {0, 0, 0}, ve, a, flxi[2] = {0, 0}, flxe[2] = {0, 0};
    const int tx = c.type_x(i - 1, j - 1), ty = c.type_y(i - 1, j - 1);
    if (tx == -1) {
        Ex[0] = 0.0;
        Ex[1] = -(ph(i + 1, j) - ph(i, j)) / c.DX(i);
    } else if (tx == 1) {
        Ex[0] = -(ph(i, j) - ph(i - 1, j)) / c.DX(i - 1);
        Ex[1] = 0.0;
    } else {
        Ex[0] = -(ph(i, j) - ph(i - 1, j)) / c.DX(i - 1);
        Ex[1] = -(ph(i + 1, j) - ph(i, j)) / c.DX(i);
    }
    if (tx == 0) {
        Te[0] = get_Te(NT(i - 1, j), NE(i - 1, j), fl);
        Te[1] = get_Te(NT(i, j), NE(i, j), fl);
        Te[2] = get_Te(NT(i + 1, j), NE(i + 1, j), fl);
        mue[0] = 5e-1 * (c.get_mue(Te[0]) + c.get_mue(Te[1]));
        mue[1] = 5e-1 * (c.get_mue(Te[1]) + c.get_mue(Te[2]));
        De[0] = 5e-1 * (c.get_De(Te[0]) + c.get_De(Te[1]));
        De[1] = 5e-1 * (c.get_De(Te[1]) + c.get_De(Te[2]));
        flxi[0] = get_flux(Ex[0], c.DX(i - 1), 1, k.mui, k.Di, NI(i - 1, j), NI(i, j));
        flxe[0] = get_flux(Ex[0], c.DX(i - 1), -1, mue[0], De[0], NE(i - 1, j), NE(i, j));
        flxi[1] = get_flux(Ex[1], c.DX(i), 1, k.mui, k.Di, NI(i, j), NI(i + 1, j));
        flxe[1] = get_flux(Ex[1], c.DX(i), -1, mue[1], De[1], NE(i, j), NE(i + 1, j));
    } else if (tx < 0) {
        Te[1] = get_Te(NT(i, j), NE(i, j), fl);
        Te[2] = get_Te(NT(i + 1, j), NE(i + 1, j), fl);
        mue[1] = 5e-1 * (c.get_mue(Te[1]) + c.get_mue(Te[2]));
        De[1] = 5e-1 * (c.get_De(Te[1]) + c.get_De(Te[2]));
        flxi[1] = get_flux(Ex[1], c.DX(i), 1, k.mui, k.Di, NI(i, j), NI(i + 1, j));
        flxe[1] = get_flux(Ex[1], c.DX(i), -1, mue[1], De[1], NE(i, j), NE(i + 1, j));
        if (tx == -2) {
            a = (ph(i - 1, j) > ph(i, j)) ? 1.0 : 0.0;
            mue[0] = c.get_mue(Te[1]);
            ve = std::sqrt((16.0 * k.e * k.ph0 * Te[1]) / (3.0 * k.pi * k.me)) * k.t0 / k.x0;
            flxi[0] = (1.0 - a) * k.mui * Ex[0] * NI(i, j) - 2.5e-1 * k.vi * NI(i, j);
            flxe[0] = -(a * mue[0] * Ex[0] * NE(i, j)) - 2.5e-1 * ve * NE(i, j) - k.gam * flxi[0];
        } else if (tx == -1) {
            flxi[0] = 0.0; flxe[0] = 0.0;
        }
    } else if (tx > 0) {
        Te[0] = get_Te(NT(i - 1, j), NE(i - 1, j), fl);
        Te[1] = get_Te(NT(i, j), NE(i, j), fl);
        mue[0] = 5e-1 * (c.get_mue(Te[0]) + c.get_mue(Te[1]));
        De[0] = 5e-1 * (c.get_De(Te[0]) + c.get_De(Te[1]));
        flxi[0] = get_flux(Ex[0], c.DX(i - 1), 1, k.mui, k.Di, NI(i - 1, j), NI(i, j));
        flxe[0] = get_flux(Ex[0], c.DX(i - 1), -1, mue[0], De[0], NE(i - 1, j), NE(i, j));
        if (tx == 2) {
            a = (ph(i + 1, j) > ph(i, j)) ? 1.0 : 0.0;
            mue[1] = c.get_mue(Te[1]);
            ve = std::sqrt((16.0 * k.e * k.ph0 * Te[1]) / (3.0 * k.pi * k.me)) * k.t0 / k.x0;
            flxi[1] = (1.0 - a) * k.mui * Ex[1] * NI(i, j) + 2.5e-1 * k.vi * NI(i, j);
            flxe[1] = -(a * mue[1] * Ex[1] * NE(i, j)) + 2.5e-1 * ve * NE(i, j) - k.gam * flxi[1];
        } else if (tx == 1) {
            flxi[1] = 0.0; flxe[1] = 0.0;
        }
    }
    dfdx = -(Ex[1] - Ex[0]) / c.DLX(i - 1);
    dflxe_x = (flxe[1] - flxe[0]) / c.DLX(i - 1);
    dflxi_x = (flxi[1] - flxi[0]) / c.DLX(i - 1);

    if (ty == -1) {
        Ey[0] = 0.0;
        Ey[1] = -(ph(i, j + 1) - ph(i, j)) / c.DY(j);
    } else if (ty == 1) {
        Ey[0] = -(ph(i, j) - ph(i, j - 1)) / c.DY(j - 1);
        Ey[1] = 0.0;
    } else if (ty == 3) {
        Ey[0] = -(ph(i, j) - ph(i, j - 1)) / c.DY(j - 1);
        Ey[1] = -c.sig_pl[i];   // sig0 = sig(i) with sig = sig_pl (lapl_lib.F90:72-76, main.F90:80)
    } else {
        Ey[0] = -(ph(i, j) - ph(i, j - 1)) / c.DY(j - 1);
        Ey[1] = -(ph(i, j + 1) - ph(i, j)) / c.DY(j);
    }
    if (ty == 0) {
        Te[0] = get_Te(NT(i, j - 1), NE(i, j - 1), fl);
        Te[1] = get_Te(NT(i, j), NE(i, j), fl);
        Te[2] = get_Te(NT(i, j + 1), NE(i, j + 1), fl);
        mue[0] = 5e-1 * (c.get_mue(Te[0]) + c.get_mue(Te[1]));
        mue[1] = 5e-1 * (c.get_mue(Te[1]) + c.get_mue(Te[2]));
        De[0] = 5e-1 * (c.get_De(Te[0]) + c.get_De(Te[1]));
        De[1] = 5e-1 * (c.get_De(Te[1]) + c.get_De(Te[2]));
        flxi[0] = get_flux(Ey[0], c.DY(j - 1), 1, k.mui, k.Di, NI(i, j - 1), NI(i, j));
        flxe[0] = get_flux(Ey[0], c.DY(j - 1), -1, mue[0], De[0], NE(i, j - 1), NE(i, j));
        flxi[1] = get_flux(Ey[1], c.DY(j), 1, k.mui, k.Di, NI(i, j), NI(i, j + 1));
        flxe[1] = get_flux(Ey[1], c.DY(j), -1, mue[1], De[1], NE(i, j), NE(i, j + 1));
    } else if (ty < 0) {
        Te[1] = get_Te(NT(i, j), NE(i, j), fl);
        Te[2] = get_Te(NT(i, j + 1), NE(i, j + 1), fl);
        mue[1] = 5e-1 * (c.get_mue(Te[1]) + c.get_mue(Te[2]));
        De[1] = 5e-1 * (c.get_De(Te[1]) + c.get_De(Te[2]));
        flxi[1] = get_flux(Ey[1], c.DY(j), 1, k.mui, k.Di, NI(i, j), NI(i, j + 1));
        flxe[1] = get_flux(Ey[1], c.DY(j), -1, mue[1], De[1], NE(i, j), NE(i, j + 1));
        flxi[0] = 0.0; flxe[0] = 0.0;
    } else if (ty > 0) {
        Te[0] = get_Te(NT(i, j - 1), NE(i, j - 1), fl);
        Te[1] = get_Te(NT(i, j), NE(i, j), fl);
        mue[0] = 5e-1 * (c.get_mue(Te[0]) + c.get_mue(Te[1]));
        De[0] = 5e-1 * (c.get_De(Te[0]) + c.get_De(Te[1]));
        flxi[0] = get_flux(Ey[0], c.DY(j - 1), 1, k.mui, k.Di, NI(i, j - 1), NI(i, j));
        flxe[0] = get_flux(Ey[0], c.DY(j - 1), -1, mue[0], De[0], NE(i, j - 1), NE(i, j));
        if (ty == 3) {
            Te[1] = get_Te(NT(i, j), NE(i, j), fl);
            mue[1] = c.get_mue(Te[1]);
            De[1] = c.get_De(Te[1]);
            flxi[1] = get_flux(Ey[1], c.DY(j), 1, k.mui, k.Di, NI(i, j), 0.0);
            flxe[1] = get_flux(Ey[1], c.DY(j), -1, mue[1], De[1], NE(i, j), 0.0);
        } else if (ty == 2) {
            a = (ph(i, j + 1) > ph(i, j)) ? 1.0 : 0.0;
            mue[1] = c.get_mue(Te[1]);
            ve = std::sqrt((16.0 * k.e * k.ph0 * Te[1]) / (3.0 * k.pi * k.me)) * k.t0 / k.x0;
            flxi[1] = (1.0 - a) * k.mui * Ey[1] * NI(i, j) + 2.5e-1 * k.vi * NI(i, j);
            flxe[1] = -(a * mue[1] * Ey[1] * NE(i, j)) + 2.5e-1 * ve * NE(i, j) - k.gam * flxi[1];
        } else {
            flxi[1] = 0.0; flxe[1] = 0.0;
        }
    }
    if (c.cfg.cyl) {
        double rp = (c.R(j + 1) + c.R(j)), rm = (c.R(j) + c.R(j - 1));
        dfdy = -(Ey[1] * rp / 2.0 - Ey[0] * rm / 2.0) / c.DLY(j - 1) / c.R(j);
        dflxi_y = (flxi[1] * rp / 2.0 - flxi[0] * rm / 2.0) / c.DLY(j - 1) / c.R(j);
        dflxe_y = (flxe[1] * rp / 2.0 - flxe[0] * rm / 2.0) / c.DLY(j - 1) / c.R(j);
    } else {
        dfdy = -(Ey[1] - Ey[0]) / c.DLY(j - 1);
        dflxi_y = (flxi[1] - flxi[0]) / c.DLY(j - 1);
        dflxe_y = (flxe[1] - flxe[0]) / c.DLY(j - 1);
    }
    double b = dfdx + dfdy + NI(i, j) - NE(i, j) - dt * (dflxi_x + dflxi_y - dflxe_x - dflxe_y);
    if (std::isnan(b)) fl.bnan = 1;   // printed only by the reference (lapl_lib.F90:376-378)
    return b;
}

// laplJ, lapl_lib.F90:381-609: row entries (west, east, south, north, centre).
void laplJ(const or_ctx &c, int i, int j, double dt, double A[5], Flags &fl) {
    const Consts &k = c.k;
    const F2 &ph = c.ph, &pm = c.ph_mi;
    auto NI = [&](int a, int b) { return c.ni(a, b, 1); };
    auto NE = [&](int a, int b) { return c.ne(a, b, 1); };
    auto NT = [&](int a, int b) { return c.nt(a, b, 1); };
    const int tx = c.type_x(i - 1, j - 1), ty = c.type_y(i - 1, j - 1);
    double E_pl, E_mi, dfxi_pl, dfxi_mi, dfxe_pl, dfxe_mi, dfyi_pl = 0, dfyi_mi = 0, dfye_pl = 0, dfye_mi = 0;
    double Te1, Te2, mue, De;
    int ac;
    for (int q = 0; q < 5; q++) A[q] = 0.0;

    if (tx >= 0) {
        Te1 = get_Te(NT(i - 1, j), NE(i - 1, j), fl);
        Te2 = get_Te(NT(i, j), NE(i, j), fl);
        mue = 5e-1 * (c.get_mue(Te1) + c.get_mue(Te2));
        De = 5e-1 * (c.get_De(Te1) + c.get_De(Te2));
        E_pl = -(ph(i, j) - ph(i - 1, j)) / c.DX(i - 1);
        E_mi = -(pm(i, j) - pm(i - 1, j)) / c.DX(i - 1);
        dfxe_mi = dfdph(E_pl, E_mi, -1, mue, De, c.DX(i - 1), NE(i - 1, j), NE(i, j), &fl);
        dfxe_mi = -(mue / c.DX(i - 1) * dfxe_mi);
        dfxi_mi = dfdph(E_pl, E_mi, 1, k.mui, k.Di, c.DX(i - 1), NI(i - 1, j), NI(i, j), &fl);
        dfxi_mi = k.mui / c.DX(i - 1) * dfxi_mi;
        A[0] = (1.0 / c.DX(i - 1) + dt * (dfxi_mi - dfxe_mi)) / c.DLX(i - 1);
    } else if (tx == -2) {
        ac = (ph(i - 1, j) > ph(i, j)) ? 1 : 0;
        Te2 = get_Te(NT(i, j), NE(i, j), fl);
        mue = c.get_mue(Te2);
        dfxi_mi = (double)(1 - ac) * k.mui * NI(i, j) / c.DX(i - 1);
        dfxe_mi = -((double)ac * mue * NE(i, j) / c.DX(i - 1)) - k.gam * dfxi_mi;
    } else {
        dfxi_mi = 0.0;
        dfxe_mi = 0.0;
    }

    if (tx <= 0) {
        Te1 = get_Te(NT(i, j), NE(i, j), fl);
        Te2 = get_Te(NT(i + 1, j), NE(i + 1, j), fl);
        mue = 5e-1 * (c.get_mue(Te1) + c.get_mue(Te2));
        De = 5e-1 * (c.get_De(Te1) + c.get_De(Te2));
        E_pl = -(ph(i + 1, j) - ph(i, j)) / c.DX(i);
        E_mi = -(pm(i + 1, j) - pm(i, j)) / c.DX(i);
        dfxe_pl = dfdph(E_pl, E_mi, -1, mue, De, c.DX(i), NE(i, j), NE(i + 1, j), &fl);
        dfxe_pl = mue / c.DX(i) * dfxe_pl;
        dfxi_pl = dfdph(E_pl, E_mi, 1, k.mui, k.Di, c.DX(i), NI(i, j), NI(i + 1, j), &fl);
        dfxi_pl = -(k.mui / c.DX(i) * dfxi_pl);
        A[1] = (1.0 / c.DX(i) - dt * (dfxi_pl - dfxe_pl)) / c.DLX(i - 1);
    } else if (tx == 2) {
        ac = (ph(i + 1, j) > ph(i, j)) ? 1 : 0;
        Te2 = get_Te(NT(i, j), NE(i, j), fl);
        mue = c.get_mue(Te2);
        dfxi_pl = (double)(ac - 1) * k.mui * NI(i, j) / c.DX(i);
        dfxe_pl = (double)ac * mue * NE(i, j) / c.DX(i) - k.gam * dfxi_pl;
    } else {
        dfxi_pl = 0.0;
        dfxe_pl = 0.0;
    }

    // ny > 1
    if (ty >= 0) {
        Te1 = get_Te(NT(i, j - 1), NE(i, j - 1), fl);
        Te2 = get_Te(NT(i, j), NE(i, j), fl);
        mue = 5e-1 * (c.get_mue(Te1) + c.get_mue(Te2));
        De = 5e-1 * (c.get_De(Te1) + c.get_De(Te2));
        E_pl = -(ph(i, j) - ph(i, j - 1)) / c.DY(j - 1);
        E_mi = -(pm(i, j) - pm(i, j - 1)) / c.DY(j - 1);
        dfye_mi = dfdph(E_pl, E_mi, -1, mue, De, c.DY(j - 1), NE(i, j - 1), NE(i, j), &fl);
        dfye_mi = -(mue / c.DY(j - 1) * dfye_mi);
        dfyi_mi = dfdph(E_pl, E_mi, 1, k.mui, k.Di, c.DY(j - 1), NI(i, j - 1), NI(i, j), &fl);
        dfyi_mi = k.mui / c.DY(j - 1) * dfyi_mi;
        if (c.cfg.cyl)
            A[2] = 5e-1 * (c.R(j) + c.R(j - 1)) / c.DY(j - 1) / c.DLY(j - 1) / c.R(j)
                 + dt * (dfyi_mi - dfye_mi) * (c.R(j) + c.R(j - 1)) / 2.0 / c.DLY(j - 1) / c.R(j);
        else
            A[2] = 1.0 / c.DY(j - 1) / c.DLY(j - 1) + dt * (dfyi_mi - dfye_mi) / c.DLY(j - 1);
    } else if (ty == -2) {
        ac = (ph(i, j - 1) > ph(i, j)) ? 1 : 0;
        Te2 = get_Te(NT(i, j), NE(i, j), fl);
        mue = c.get_mue(Te2);
        dfyi_mi = (double)(1 - ac) * k.mui * NI(i, j) / c.DY(j - 1);
        dfye_mi = -((double)ac * mue * NE(i, j) / c.DY(j - 1)) - k.gam * dfyi_mi;
    } else {
        dfyi_mi = 0.0;
        dfye_mi = 0.0;
    }
    if (ty <= 0) {
        Te1 = get_Te(NT(i, j), NE(i, j), fl);
        Te2 = get_Te(NT(i, j + 1), NE(i, j + 1), fl);
        mue = 5e-1 * (c.get_mue(Te1) + c.get_mue(Te2));
        De = 5e-1 * (c.get_De(Te1) + c.get_De(Te2));
        E_pl = -(ph(i, j + 1) - ph(i, j)) / c.DY(j);
        E_mi = -(pm(i, j + 1) - pm(i, j)) / c.DY(j);
        dfye_pl = dfdph(E_pl, E_mi, -1, mue, De, c.DY(j), NE(i, j), NE(i, j + 1), &fl);
        dfye_pl = mue / c.DY(j) * dfye_pl;
        dfyi_pl = dfdph(E_pl, E_mi, 1, k.mui, k.Di, c.DY(j), NI(i, j), NI(i, j + 1), &fl);
        dfyi_pl = -(k.mui / c.DY(j) * dfyi_pl);
        if (c.cfg.cyl)
            A[3] = 5e-1 * (c.R(j + 1) + c.R(j)) / c.DY(j) / c.DLY(j - 1) / c.R(j)
                 - dt * (dfyi_pl - dfye_pl) * (c.R(j + 1) + c.R(j)) / 2.0 / c.DLY(j - 1) / c.R(j);
        else
            A[3] = 1.0 / c.DY(j) / c.DLY(j - 1) - dt * (dfyi_pl - dfye_pl) / c.DLY(j - 1);
    } else if (ty == 2) {
        ac = (ph(i, j + 1) > ph(i, j)) ? 1 : 0;
        Te2 = get_Te(NT(i, j), NE(i, j), fl);
        mue = c.get_mue(Te2);
        dfyi_pl = (double)(ac - 1) * k.mui * NI(i, j) / c.DY(j);
        dfye_pl = (double)ac * mue * NE(i, j) / c.DY(j) - k.gam * dfyi_pl;
    } else {
        dfyi_pl = 0.0;   // type_y == 3 sets both to zero as well (:548-559)
        dfye_pl = 0.0;
    }

    double Ac = dt * (dfxi_pl - dfxi_mi - dfxe_pl + dfxe_mi) / c.DLX(i - 1);
    if (tx == -1) Ac = Ac - 1.0 / c.DX(i - 1) / c.DLX(i - 1);
    else if (tx == 1) Ac = Ac - 1.0 / c.DX(i - 1) / c.DLX(i - 1);
    else Ac = Ac - 1.0 / c.DLX(i - 1) * (1.0 / c.DX(i) + 1.0 / c.DX(i - 1));
    if (c.cfg.cyl)
        Ac = Ac + dt * ((dfyi_pl - dfye_pl) * (c.R(j + 1) + c.R(j)) / 2.0
                        - (dfyi_mi - dfye_mi) * (c.R(j) + c.R(j - 1)) / 2.0) / c.DLY(j - 1) / c.R(j);
    else
        Ac = Ac + dt * (dfyi_pl - dfyi_mi - dfye_pl + dfye_mi) / c.DLY(j - 1);
    if (ty == -1) {
        if (c.cfg.cyl) Ac = Ac - 1.0 / c.DY(j - 1) / c.DLY(j - 1) * (c.R(j + 1) + c.R(j)) / 2.0 / c.R(j);
        else Ac = Ac - 1.0 / c.DY(j - 1) / c.DLY(j - 1);
    } else if (ty == 1) {
        if (c.cfg.cyl) Ac = Ac - 1.0 / c.DY(j - 1) / c.DLY(j - 1) * (c.R(j) + c.R(j - 1)) / 2.0 / c.R(j);
        else Ac = Ac - 1.0 / c.DY(j - 1) / c.DLY(j - 1);
    } else {
        if (c.cfg.cyl)
            Ac = Ac - 5e-1 * ((c.R(j + 1) + c.R(j)) / c.DY(j) + (c.R(j) + c.R(j - 1)) / c.DY(j - 1))
                      / c.DLY(j - 1) / c.R(j);
        else Ac = Ac - 1.0 / c.DLY(j - 1) * (1.0 / c.DY(j) + 1.0 / c.DY(j - 1));
    }
    A[4] = Ac;
}

// ---------------- sparse 5-point matrix on interior nodes n = (i-2)+(j-2)*bx
struct Sys {
    int bx, by;
    size_t N;
    std::vector<double> w, e, s, nn, c;   // row entries (0 where absent)
    double mv(const std::vector<double> &x, size_t q) const {
        int i = (int)(q % bx), j = (int)(q / bx);
        double v = c[q] * x[q];
        if (i > 0) v += w[q] * x[q - 1];
        if (i < bx - 1) v += e[q] * x[q + 1];
        if (j > 0) v += s[q] * x[q - bx];
        if (j < by - 1) v += nn[q] * x[q + bx];
        return v;
    }
};

int nthreads_now() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// deterministic parallel dot product: fixed per-thread chunks, summed in order
double pdot(const std::vector<double> &a, const std::vector<double> &b) {
    int T = nthreads_now();
    size_t N = a.size();
    std::vector<double> part(T, 0.0);
#pragma omp parallel num_threads(T)
    {
#ifdef _OPENMP
        int t = omp_get_thread_num();
#else
        int t = 0;
#endif
        size_t lo = N * t / T, hi = N * (t + 1) / T;
        double s = 0.0;
        for (size_t q = lo; q < hi; q++) s += a[q] * b[q];
        part[t] = s;
    }
    double s = 0.0;
    for (int t = 0; t < T; t++) s += part[t];
    return s;
}

// banded LU without pivoting (bandwidth bx), exact to rounding
int solve_direct(const Sys &A, const std::vector<double> &rhs, std::vector<double> &x) {
    const int bw = A.bx;
    const size_t N = A.N;
    const int W = 2 * bw + 1;
    std::vector<double> band((size_t)W * N, 0.0);   // band[(q - p + bw) + p*W] = A(q, p)? row-major rows
    auto B = [&](size_t row, size_t col) -> double & { return band[row * W + (col + bw - row)]; };
    for (size_t q = 0; q < N; q++) {
        int i = (int)(q % A.bx), j = (int)(q / A.bx);
        B(q, q) = A.c[q];
        if (i > 0) B(q, q - 1) = A.w[q];
        if (i < A.bx - 1) B(q, q + 1) = A.e[q];
        if (j > 0) B(q, q - A.bx) = A.s[q];
        if (j < A.by - 1) B(q, q + A.bx) = A.nn[q];
    }
    x = rhs;
    for (size_t k = 0; k < N; k++) {
        double piv = B(k, k);
        if (piv == 0.0 || std::isnan(piv)) return 1;
        size_t rend = std::min(N, k + (size_t)bw + 1);
        size_t cend = std::min(N, k + (size_t)bw + 1);
        for (size_t r = k + 1; r < rend; r++) {
            double l = B(r, k);
            if (l == 0.0) continue;
            l /= piv;
            B(r, k) = l;
            for (size_t cc = k + 1; cc < cend; cc++) B(r, cc) -= l * B(k, cc);
            x[r] -= l * x[k];
        }
    }
    for (size_t kk = N; kk-- > 0;) {
        double s = x[kk];
        size_t cend = std::min(N, kk + (size_t)bw + 1);
        for (size_t cc = kk + 1; cc < cend; cc++) s -= B(kk, cc) * x[cc];
        x[kk] = s / B(kk, kk);
        if (std::isnan(x[kk])) return 1;
    }
    return 0;
}

// BiCGStab (right preconditioned) + block-Jacobi ILU(0), one block of rows per thread
int solve_bicgstab(const Sys &A, const std::vector<double> &rhs, std::vector<double> &x,
                   double rtol, int maxit, int &iters, double &relres) {
    const size_t N = A.N;
    const int bx = A.bx;
    int T = nthreads_now();
    int nb = std::max(1, std::min(T, A.by));
    std::vector<int> jlo(nb + 1);
    for (int b = 0; b <= nb; b++) jlo[b] = (int)((long)A.by * b / nb);
    std::vector<int> blk(A.by);
    for (int b = 0; b < nb; b++) for (int j = jlo[b]; j < jlo[b + 1]; j++) blk[j] = b;
    // ILU(0) pivots
    std::vector<double> d(N);
#pragma omp parallel for schedule(static, 1)
    for (int b = 0; b < nb; b++)
        for (int j = jlo[b]; j < jlo[b + 1]; j++)
            for (int i = 0; i < bx; i++) {
                size_t q = (size_t)i + (size_t)j * bx;
                double v = A.c[q];
                if (i > 0) v -= A.w[q] * A.e[q - 1] / d[q - 1];
                if (j > jlo[b]) v -= A.s[q] * A.nn[q - bx] / d[q - bx];
                d[q] = v;
            }
    auto precond = [&](const std::vector<double> &r, std::vector<double> &z) {
#pragma omp parallel for schedule(static, 1)
        for (int b = 0; b < nb; b++) {
            for (int j = jlo[b]; j < jlo[b + 1]; j++)
                for (int i = 0; i < bx; i++) {
                    size_t q = (size_t)i + (size_t)j * bx;
                    double v = r[q];
                    if (i > 0) v -= A.w[q] * z[q - 1];
                    if (j > jlo[b]) v -= A.s[q] * z[q - bx];
                    z[q] = v / d[q];
                }
            for (int j = jlo[b + 1] - 1; j >= jlo[b]; j--)
                for (int i = bx - 1; i >= 0; i--) {
                    size_t q = (size_t)i + (size_t)j * bx;
                    double v = 0.0;
                    if (i < bx - 1) v += A.e[q] * z[q + 1];
                    if (j < jlo[b + 1] - 1) v += A.nn[q] * z[q + bx];
                    z[q] = z[q] - v / d[q];
                }
        }
    };
    auto matvec = [&](const std::vector<double> &v, std::vector<double> &out) {
#pragma omp parallel for schedule(static)
        for (long q = 0; q < (long)N; q++) out[q] = A.mv(v, (size_t)q);
    };
    x.assign(N, 0.0);
    std::vector<double> r = rhs, rh = rhs, p(N, 0.0), v(N, 0.0), ph(N), s(N), sh(N), t(N);
    double bnorm = std::sqrt(pdot(rhs, rhs));
    iters = 0;
    if (bnorm == 0.0) { relres = 0.0; return 0; }
    double rho = 1, alpha = 1, omega = 1;
    for (int it = 1; it <= maxit; it++) {
        iters = it;
        double rho_n = pdot(rh, r);
        if (rho_n == 0.0 || std::isnan(rho_n)) { relres = std::sqrt(pdot(r, r)) / bnorm; return 1; }
        double beta = (rho_n / rho) * (alpha / omega);
#pragma omp parallel for schedule(static)
        for (long q = 0; q < (long)N; q++) p[q] = r[q] + beta * (p[q] - omega * v[q]);
        precond(p, ph);
        matvec(ph, v);
        alpha = rho_n / pdot(rh, v);
#pragma omp parallel for schedule(static)
        for (long q = 0; q < (long)N; q++) s[q] = r[q] - alpha * v[q];
        double sn = std::sqrt(pdot(s, s)) / bnorm;
        if (sn <= rtol) {
#pragma omp parallel for schedule(static)
            for (long q = 0; q < (long)N; q++) x[q] += alpha * ph[q];
            relres = sn;
            return 0;
        }
        precond(s, sh);
        matvec(sh, t);
        double tt = pdot(t, t);
        omega = tt > 0 ? pdot(t, s) / tt : 0.0;
#pragma omp parallel for schedule(static)
        for (long q = 0; q < (long)N; q++) {
            x[q] += alpha * ph[q] + omega * sh[q];
            r[q] = s[q] - omega * t[q];
        }
        rho = rho_n;
        double rn = std::sqrt(pdot(r, r)) / bnorm;
        relres = rn;
        if (std::isnan(rn)) return 1;
        if (rn <= rtol) return 0;
        if (omega == 0.0) return 1;
    }
    return 1;
}

void assemble(const or_ctx &c, double dt, Sys &S, std::vector<double> &b, Flags &fl) {
    const int bx = c.bx, by = c.by;
    S.bx = bx; S.by = by; S.N = (size_t)bx * by;
    S.w.assign(S.N, 0); S.e.assign(S.N, 0); S.s.assign(S.N, 0); S.nn.assign(S.N, 0); S.c.assign(S.N, 0);
    b.assign(S.N, 0);
    std::vector<Flags> fls(by + 2);
#pragma omp parallel for schedule(static)
    for (int j = 2; j <= by + 1; j++)
        for (int i = 2; i <= bx + 1; i++) {
            size_t q = (size_t)(i - 2) + (size_t)(j - 2) * bx;
            double A[5];
            b[q] = laplEqn(c, i, j, dt, fls[j]);
            laplJ(c, i, j, dt, A, fls[j]);
            S.w[q] = A[0]; S.e[q] = A[1]; S.s[q] = A[2]; S.nn[q] = A[3]; S.c[q] = A[4];
        }
    for (int j = 2; j <= by + 1; j++) { fl.neg |= fls[j].neg; fl.nan |= fls[j].nan; fl.bnan |= fls[j].bnan; }
}

// lapl_solve, lapl_lib.F90:57-121
int lapl_solve(or_ctx &c, double dt, int &lerr, int &iters, double &relres) {
    Sys S;
    std::vector<double> b;
    Flags fl;
    assemble(c, dt, S, b, fl);
    if (fl.neg) { c.err = "negative density in get_Te"; return FS_ERR_NEG_DENSITY; }
    // dFdPh stops on NaN (lapl_lib.F90:632-635); a NaN right-hand side makes the
    // Krylov solve diverge, which the reference reports as lerr = 1 (:104-109)
    if (fl.nan) { c.err = "NaN in dFdPh"; return FS_ERR_NAN; }
    if (fl.bnan) { lerr = 1; iters = 0; relres = NAN; return FS_OK; }
    std::vector<double> rhs(S.N), x;
    for (size_t q = 0; q < S.N; q++) rhs[q] = -b[q];
    int conv_fail;
    iters = 0;
    if (c.solver == OR_SOLVER_DIRECT) {
        conv_fail = solve_direct(S, rhs, x);
        iters = 1;
        double rn = 0, bn = 0;
        for (size_t q = 0; q < S.N; q++) {
            double rr = S.mv(x, q) - rhs[q];
            rn += rr * rr;
            bn += rhs[q] * rhs[q];
        }
        relres = bn > 0 ? std::sqrt(rn / bn) : 0.0;
    } else {
        conv_fail = solve_bicgstab(S, rhs, x, c.cfg.lapl_rtol, c.cfg.lapl_maxit, iters, relres);
    }
    if (conv_fail) {
        lerr = 1;
        return FS_OK;
    }
    lerr = 0;
    for (int j = 2; j <= c.by + 1; j++)
        for (int i = 2; i <= c.bx + 1; i++)
            c.ph(i, j) = c.ph(i, j) + x[(size_t)(i - 2) + (size_t)(j - 2) * c.bx];
    c.ph_mi = c.ph;
    return FS_OK;
}

void rotate_accept(or_ctx &c) {    // main.F90:83-101
    c.ts++;
    c.t = c.t + c.dt;
    F3 *sp[4] = {&c.ni, &c.ne, &c.nm, &c.nt};
    for (F3 *s : sp) {
        if (s == &c.nm && c.cfg.nspecies != 4) continue;
        s->copy_level(3, 2);
        s->copy_level(2, 1);
    }
    c.Vd_or = c.Vd_mi;
    c.Vd_mi = c.Vd_pl;
    c.sig_or = c.sig_mi;
    c.sig_mi = c.sig_pl;
}

void rotate_reject(or_ctx &c) {    // main.F90:103-121
    c.dt = c.dt / 2.0;
    F3 *sp[4] = {&c.ni, &c.ne, &c.nm, &c.nt};
    for (F3 *s : sp) {
        if (s == &c.nm && c.cfg.nspecies != 4) continue;
        s->copy_level(1, 3);
        s->copy_level(2, 3);
    }
    c.Vd_pl = c.Vd_or;
    c.Vd_mi = c.Vd_or;
    c.sig_pl = c.sig_or;
    c.sig_mi = c.sig_or;
}

}  // namespace

// ============================================================== C interface
extern "C" {

int or_get_constants(const fs_config *cfg, fs_constants *o) {
    if (!cfg || !o) return FS_ERR_INVALID;
    Consts k = make_consts(*cfg);
    o->pi = k.pi; o->eps0 = k.eps0; o->e = k.e; o->kb = k.kb; o->me = k.me; o->x0 = k.x0;
    o->ph0 = k.ph0; o->t0 = k.t0; o->wp02 = k.wp02; o->w2 = k.w2; o->tg = k.tg; o->p = k.p;
    o->ninf = k.ninf; o->n_zero = k.n_zero; o->mi = k.mi; o->mui = k.mui; o->vi = k.vi;
    o->Di = k.Di; o->Dm = k.Dm; o->k_r = k.k_r; o->k_mp = k.k_mp; o->k_2q = k.k_2q;
    o->k_3q = k.k_3q; o->h_ir = k.h_ir; o->h_ex = k.h_ex; o->h_si = k.h_si; o->h_sc = k.h_sc;
    o->gam = k.gam; o->nmin_nt = k.n_zero / k.ph0 / 1e2; o->cap = k.cap;
    return FS_OK;
}

int or_build_table(const fs_config *cfg, double *out) {
    if (!cfg || !out || cfg->table_n < 2) return FS_ERR_INVALID;
    Consts k = make_consts(*cfg);
    Table t;
    t.build(*cfg, k);
    std::memcpy(out, t.v.data(), sizeof(double) * t.v.size());
    return FS_OK;
}

int or_set_threads(int32_t n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

int or_create(const fs_config *cfg, const fs_mesh *m, int32_t solver, or_ctx **out) {
    if (!cfg || !m || !out) { g_create_error = "null argument"; return FS_ERR_INVALID; }
    if (cfg->abi_version != FS_ABI_VERSION) { g_create_error = "ABI version mismatch"; return FS_ERR_INVALID; }
    if (cfg->nx < 3 || cfg->ny < 2) { g_create_error = "grid must have nx >= 3 and ny >= 2"; return FS_ERR_UNSUPPORTED; }
    if (cfg->nspecies != 3 && cfg->nspecies != 4) { g_create_error = "nspecies must be 3 or 4"; return FS_ERR_INVALID; }
    if (cfg->rf < 0 || cfg->rf > 3) { g_create_error = "rf must be 0 (DC), 1 (AC), 2 or 3 (pulses)"; return FS_ERR_UNSUPPORTED; }
    if (cfg->rf == 1 && !(cfg->res > 0)) { g_create_error = "the AC source needs res > 0"; return FS_ERR_INVALID; }
    if (cfg->coef_mode == FS_COEF_TABLE && cfg->table_n < 2) { g_create_error = "table_n < 2"; return FS_ERR_INVALID; }
    or_ctx *c = new or_ctx();
    c->cfg = *cfg;
    c->k = make_consts(*cfg);
    if (cfg->coef_mode == FS_COEF_TABLE) c->tab.build(*cfg, c->k);
    c->nx = c->bx = cfg->nx;
    c->ny = c->by = cfg->ny;
    c->solver = solver;
    const int bx = c->bx, by = c->by;
    c->dx.assign(bx + 2, 0); c->dlx.assign(bx + 1, 0); c->dy.assign(by + 2, 0); c->dly.assign(by + 1, 0);
    c->r.assign(by + 3, 0);
    for (int i = 1; i <= bx + 1; i++) c->dx[i] = m->dx[i - 1];
    for (int i = 1; i <= bx; i++) c->dlx[i] = m->dlx[i - 1];
    for (int j = 1; j <= by + 1; j++) c->dy[j] = m->dy[j - 1];
    for (int j = 1; j <= by; j++) c->dly[j] = m->dly[j - 1];
    for (int j = 1; j <= by + 2; j++) c->r[j] = m->r[j - 1];
    c->tx.assign(m->type_x, m->type_x + (size_t)bx * by);
    c->ty.assign(m->type_y, m->type_y + (size_t)bx * by);
    const int ld = bx + 2;
    // ptcl_init (ptcl_lib.F90:15-30)
    c->ki.init(ld, by + 2, 5); c->ke.init(ld, by + 2, 5); c->kt.init(ld, by + 2, 5); c->km.init(ld, by + 2, 5);
    c->ni.init(ld, by + 2, 3, cfg->n_init);
    c->ne.init(ld, by + 2, 3, cfg->n_init);
    c->nt.init(ld, by + 2, 3, cfg->n_init * c->k.tg * c->k.kb / c->k.e / c->k.ph0);
    c->nm.init(ld, by + 2, 3, cfg->n_init);
    // lapl_init
    c->ph.init(ld, by + 2, 0.0);
    c->ph_mi.init(ld, by + 2, 0.0);
    // circ_init
    c->Vmax = c->Vsrc = c->Vd_pl = c->Vd_mi = c->Vd_or = cfg->vl;
    // sfc_init (sfc_lib.F90:84-90); rwall is on when the mesh has wall nodes
    c->sig_pl.assign(bx + 3, 0.0); c->sig_mi.assign(bx + 3, 0.0); c->sig_or.assign(bx + 3, 0.0);
    c->ks.assign((size_t)(bx + 3) * 5, 0.0);
    for (int q : c->ty) c->rwall = c->rwall || q == 3;
    std::memset(&c->st, 0, sizeof(c->st));
    *out = c;
    return FS_OK;
}

void or_destroy(or_ctx *c) { delete c; }

const char *or_last_error(const or_ctx *c) { return c ? c->err.c_str() : g_create_error.c_str(); }

int or_set_time(or_ctx *c, double t, double dt) { c->t = t; c->dt = dt; return FS_OK; }

int or_get_controller(or_ctx *c, double *err_prev, int64_t *ts) {
    if (err_prev) *err_prev = c->err_prev;
    if (ts) *ts = c->ts;
    return FS_OK;
}

int or_set_controller(or_ctx *c, double err_prev, int64_t ts) {
    c->err_prev = err_prev;
    c->ts = ts;
    return FS_OK;
}

static void copy_in(F3 &f, const double *src, int ld, int nlev, int bx, int by) {
    for (int l = 1; l <= 3; l++) {
        int sl = nlev == 1 ? 1 : l;
        for (int j = 1; j <= by + 2; j++)
            for (int i = 1; i <= bx + 2; i++)
                f(i, j, l) = src[(size_t)(i - 1) + ((size_t)(j - 1) + (size_t)(sl - 1) * (by + 2)) * ld];
    }
}
static void copy_out(const F3 &f, double *dst, int ld, int nlev, int bx, int by) {
    for (int l = 1; l <= nlev; l++)
        for (int j = 1; j <= by + 2; j++)
            for (int i = 1; i <= bx + 2; i++)
                dst[(size_t)(i - 1) + ((size_t)(j - 1) + (size_t)(l - 1) * (by + 2)) * ld] = f(i, j, l);
}

int or_upload_state(or_ctx *c, const double *ni, const double *ne, const double *nt,
                    const double *nm, const double *ph, int32_t ld, int32_t nlev) {
    if (ld < c->bx + 2 || (nlev != 1 && nlev != 3)) return FS_ERR_INVALID;
    if (ni) copy_in(c->ni, ni, ld, nlev, c->bx, c->by);
    if (ne) copy_in(c->ne, ne, ld, nlev, c->bx, c->by);
    if (nt) copy_in(c->nt, nt, ld, nlev, c->bx, c->by);
    if (nm) copy_in(c->nm, nm, ld, nlev, c->bx, c->by);
    if (ph) {
        for (int j = 1; j <= c->by + 2; j++)
            for (int i = 1; i <= c->bx + 2; i++) c->ph(i, j) = ph[(size_t)(i - 1) + (size_t)(j - 1) * ld];
        c->ph_mi = c->ph;
    }
    return FS_OK;
}

int or_download_state(or_ctx *c, double *ni, double *ne, double *nt, double *nm,
                      double *ph, int32_t ld, int32_t nlev) {
    if (ld < c->bx + 2 || (nlev != 1 && nlev != 3)) return FS_ERR_INVALID;
    if (ni) copy_out(c->ni, ni, ld, nlev, c->bx, c->by);
    if (ne) copy_out(c->ne, ne, ld, nlev, c->bx, c->by);
    if (nt) copy_out(c->nt, nt, ld, nlev, c->bx, c->by);
    if (nm) copy_out(c->nm, nm, ld, nlev, c->bx, c->by);
    if (ph)
        for (int j = 1; j <= c->by + 2; j++)
            for (int i = 1; i <= c->bx + 2; i++) ph[(size_t)(i - 1) + (size_t)(j - 1) * ld] = c->ph(i, j);
    return FS_OK;
}

int or_download_k(or_ctx *c, double *ki, double *ke, double *kt, double *km, int32_t ld) {
    if (ld < c->bx + 2) return FS_ERR_INVALID;
    F3 *src[4] = {&c->ki, &c->ke, &c->kt, &c->km};
    double *dst[4] = {ki, ke, kt, km};
    for (int s = 0; s < 4; s++) {
        if (!dst[s]) continue;
        for (int l = 1; l <= 5; l++)
            for (int j = 1; j <= c->by + 2; j++)
                for (int i = 1; i <= c->bx + 2; i++)
                    dst[s][(size_t)(i - 1) + ((size_t)(j - 1) + (size_t)(l - 1) * (c->by + 2)) * ld] = (*src[s])(i, j, l);
    }
    return FS_OK;
}

int or_ptcl_step(or_ctx *c, double *dt_inout, double *t_m_out, double *ida_out,
                 double *idc_out, int32_t *attempts_out) {
    if (dt_inout) c->dt = *dt_inout;
    c->t_m = 1e9;
    int attempts = 0;
    int rc = ptcl_step(*c, attempts);
    c->st.attempts += attempts;
    if (dt_inout) *dt_inout = c->dt;
    if (t_m_out) *t_m_out = c->t_m;
    if (ida_out) *ida_out = c->Ida;
    if (idc_out) *idc_out = c->Idc;
    if (attempts_out) *attempts_out = attempts;
    return rc;
}

int or_lapl_solve(or_ctx *c, double dt, int32_t *lerr_out, int32_t *iters_out, double *relres_out) {
    int lerr = 0, iters = 0;
    double relres = 0;
    int rc = lapl_solve(*c, dt, lerr, iters, relres);
    c->st.lapl_iters += iters;
    c->st.last_lapl_iters = iters;
    c->st.lapl_relres = relres;
    c->st.lerr = lerr;
    if (lerr_out) *lerr_out = lerr;
    if (iters_out) *iters_out = iters;
    if (relres_out) *relres_out = relres;
    return rc;
}

int or_lapl_assemble(or_ctx *c, double dt, double *b, double *a5) {
    Sys S;
    std::vector<double> bb;
    Flags fl;
    assemble(*c, dt, S, bb, fl);
    for (size_t q = 0; q < S.N; q++) {
        if (b) b[q] = bb[q];
        if (a5) {
            a5[5 * q + 0] = S.w[q]; a5[5 * q + 1] = S.e[q]; a5[5 * q + 2] = S.s[q];
            a5[5 * q + 3] = S.nn[q]; a5[5 * q + 4] = S.c[q];
        }
    }
    if (fl.neg) return FS_ERR_NEG_DENSITY;
    if (fl.nan) return FS_ERR_NAN;
    return FS_OK;
}

int or_get_surface_charge(or_ctx *c, double *sig_pl, double *sig_mi, double *sig_or) {
    const std::vector<double> *src[3] = {&c->sig_pl, &c->sig_mi, &c->sig_or};
    double *dst[3] = {sig_pl, sig_mi, sig_or};
    for (int q = 0; q < 3; q++)
        if (dst[q]) std::memcpy(dst[q], src[q]->data() + 1, sizeof(double) * (c->bx + 2));
    return FS_OK;
}

int or_set_surface_charge(or_ctx *c, const double *sig_pl, const double *sig_mi, const double *sig_or) {
    std::vector<double> *dst[3] = {&c->sig_pl, &c->sig_mi, &c->sig_or};
    const double *src[3] = {sig_pl, sig_mi, sig_or};
    for (int q = 0; q < 3; q++)
        if (src[q]) std::memcpy(dst[q]->data() + 1, src[q], sizeof(double) * (c->bx + 2));
    return FS_OK;
}

int or_get_circuit(or_ctx *c, double *v) {
    v[0] = c->Vd_pl; v[1] = c->Vd_mi; v[2] = c->Vd_or; v[3] = c->Vsrc;
    return FS_OK;
}

int or_set_circuit(or_ctx *c, const double *v) {
    c->Vd_pl = v[0]; c->Vd_mi = v[1]; c->Vd_or = v[2];
    return FS_OK;
}

int or_accept(or_ctx *c) { rotate_accept(*c); return FS_OK; }
int or_reject(or_ctx *c) { rotate_reject(*c); return FS_OK; }

int or_run(or_ctx *c, int32_t nsteps, fs_stats *out) {
    for (int s = 0; s < nsteps; s++) {
        c->t_m = 1e9;
        if (c->ts > 1) {
            int att = 0;
            int rc = ptcl_step(*c, att);
            c->st.attempts += att;
            if (rc) return rc;
        }
        int lerr = 0, iters = 0;
        double relres = 0;
        int rc = lapl_solve(*c, c->dt, lerr, iters, relres);
        if (rc) return rc;
        c->st.lapl_iters += iters;
        c->st.last_lapl_iters = iters;
        c->st.lapl_relres = relres;
        c->st.lerr = lerr;
        if (lerr == 0) rotate_accept(*c);
        else { rotate_reject(*c); c->st.lapl_rejects++; }
    }
    return or_get_stats(c, out);
}

int or_get_stats(or_ctx *c, fs_stats *out) {
    if (!out) return FS_OK;
    c->st.t = c->t;
    c->st.dt = c->dt;
    c->st.t_m = c->t_m;
    c->st.ida = c->Ida;
    c->st.idc = c->Idc;
    c->st.err_cur = c->err_cur;
    c->st.dt_step = c->dt_step;
    c->st.steps = c->ts;
    *out = c->st;
    return FS_OK;
}

double or_get_flux(double E, double dh, int32_t q, double mu, double D, double nl, double nr) {
    return get_flux(E, dh, q, mu, D, nl, nr);
}

double or_dfdph(double E_pl, double E_mi, int32_t q, double mu, double D, double dx,
                double n1, double n2) {
    return dfdph(E_pl, E_mi, q, mu, D, dx, n1, n2, nullptr);
}

double or_coef(const or_ctx *c, int32_t which, double T) {
    if (which == 8) return c->get_mut(T);
    if (which == 9) return c->get_Dt(T);
    return c->coef(which, T);
}

}  // extern "C"
