// fs_fits.h -- the reference's local-mean-energy coefficient fits
// (ptcl_props.F90:182-429), evaluated at the nondimensional mean energy T on
// the host (to fill the coefficient table) and on the device (the per-node
// fit mode, FS_COEF_FITS).  Literals the reference writes without a d
// exponent are REAL(4) and are rounded through float (FS_F32); x**n with
// integer n is a multiplication chain, as gfortran evaluates it.
#pragma once
#include <cmath>
#include <cuda_runtime.h>

#include "../../include/fluidsim_gpu.h"

#define FS_HD __host__ __device__ __forceinline__
#define FS_F32(v) ((double)(v))

struct FitEval {
    double ph0, x0, t0, x03, ninf;
    // branch points of the piecewise fits, REAL(4) logarithms evaluated on the
    // host (fs_fit_eval) so that host and device branch identically
    double th_mue, th_kex, th_kir;
    FS_HD static double q2(double x) { return x * x; }
    FS_HD static double q3(double x) { return q2(x) * x; }
    FS_HD static double q4(double x) { double t = q2(x); return t * t; }
    FS_HD static double q5(double x) { return q3(x) * q2(x); }
    FS_HD static double q6(double x) { double t = q3(x); return t * t; }
    FS_HD static double q7(double x) { return q4(x) * q3(x); }
    FS_HD static double q8(double x) { double t = q4(x); return t * t; }
    FS_HD static double q9(double x) { return q6(x) * q3(x); }
    FS_HD static double q10(double x) { double t = q5(x); return t * t; }
    FS_HD static double q11(double x) { return q6(x) * q5(x); }
    FS_HD double clog(double lo, double hi, double T) const { return log(fmax(lo, fmin(hi, T * ph0))); }

    FS_HD double mue(double T) const {
        double x = clog(2.34e-1, 1.57e2, T), s;
        if (x < th_mue)
            s = FS_F32(58.1133016145f) + FS_F32(-0.984082217962f) * x + FS_F32(-0.164770900119f) * q2(x)
              + FS_F32(-0.142058042584f) * q3(x) + FS_F32(-0.0637079234081f) * q4(x) + FS_F32(0.0436642742558f) * q5(x);
        else
            s = FS_F32(70.7846754548f) + FS_F32(-22.7558138237f) * x + FS_F32(12.8366493242f) * q2(x)
              + FS_F32(-3.57242763244f) * q3(x) + FS_F32(0.486276623664f) * q4(x) + FS_F32(-0.0259045697422f) * q5(x);
        return exp(s) * x0 / ninf * t0 * ph0;
    }
    // get_mut (ptcl_props.F90:223-250): same range and branch point as get_mue
    FS_HD double mut(double T) const {
        double x = clog(2.34e-1, 1.57e2, T), s;
        if (x < th_mue)
            s = FS_F32(58.1354622038f) + FS_F32(-1.29918391109f) * x + FS_F32(-0.106559658509f) * q2(x)
              + FS_F32(-0.0202265418394f) * q3(x) + FS_F32(-0.0286667333915f) * q4(x) + FS_F32(0.022457210094f) * q5(x);
        else
            s = FS_F32(68.2627663433f) + FS_F32(-19.3524000831f) * x + FS_F32(11.3251980583f) * q2(x)
              + FS_F32(-3.24070386509f) * q3(x) + FS_F32(0.449848156054f) * q4(x) + FS_F32(-0.0242585762405f) * q5(x);
        return exp(s) * x0 / ninf * t0 * ph0;
    }
    // get_Dt (ptcl_props.F90:293-316)
    FS_HD double Dt(double T) const {
        double x = clog(2.34e-1, 1.57e2, T);
        double s = FS_F32(57.7214952841f) + FS_F32(-0.353731464348f) * x + FS_F32(-0.00505156731795f) * q2(x)
                 + FS_F32(0.161173720584f) * q3(x) + FS_F32(-0.196610345869f) * q4(x) + FS_F32(-0.0719115643218f) * q5(x)
                 + FS_F32(0.11874085868f) * q6(x) + FS_F32(-0.00669712724784f) * q7(x) + FS_F32(-0.0236445308504f) * q8(x)
                 + FS_F32(0.00917326671764f) * q9(x) + FS_F32(-0.00135453096483f) * q10(x) + FS_F32(7.26379684461e-05f) * q11(x);
        return exp(s) * x0 / ninf * t0;
    }
    FS_HD double De(double T) const {
        double x = clog(2.34e-1, 1.57e2, T);
        double s = FS_F32(57.7067018813f) + FS_F32(-0.0699892875381f) * x + FS_F32(-0.117645585949f) * q2(x)
                 + FS_F32(0.105390295278f) * q3(x) + FS_F32(-0.102862612604f) * q4(x) + FS_F32(-0.0469171521686f) * q5(x)
                 + FS_F32(0.0584908312121f) * q6(x) + FS_F32(0.000578601715687f) * q7(x) + FS_F32(-0.0122860884883f) * q8(x)
                 + FS_F32(0.00426793748856f) * q9(x) + FS_F32(-0.000590000082557f) * q10(x) + FS_F32(3.00706533201e-05f) * q11(x);
        return exp(s) * x0 / ninf * t0;
    }
    FS_HD double k_ex(double T) const {
        double x = clog(9.611e-1, 1.57e2, T), s;
        if (x < th_kex)
            s = FS_F32(-54.4513453969f) + FS_F32(17.1472529739f) * x + FS_F32(-1.05188982824f) * q2(x)
              + FS_F32(-10.5053010711f) * q3(x) + FS_F32(7.51502551486f) * q4(x) + FS_F32(-1.44763942525f) * q5(x);
        else
            s = FS_F32(-150.266369415f) + FS_F32(158.67012941f) * x + FS_F32(-85.5163470769f) * q2(x)
              + FS_F32(23.0655081891f) * q3(x) + FS_F32(-3.0908688844f) * q4(x) + FS_F32(0.16403226902f) * q5(x);
        return exp(s) * t0 / x03;
    }
    FS_HD double k_ir_fit(double T) const {
        double x = clog(1.37, 1.57e2, T), s;
        if (x < th_kir)
            s = FS_F32(-73.27080258f) + FS_F32(-30.1312514721f) * x + FS_F32(138.743842326f) * q2(x)
              + FS_F32(-161.378167125f) * q3(x) + FS_F32(81.9325486193f) * q4(x) + FS_F32(-14.9080865672f) * q5(x);
        else
            s = FS_F32(-168.925304837f) + FS_F32(177.113452524f) * x + FS_F32(-92.3047166553f) * q2(x)
              + FS_F32(24.1814225482f) * q3(x) + FS_F32(-3.15463258104f) * q4(x) + FS_F32(0.16331188192f) * q5(x);
        return exp(s) * t0 / x03;
    }
    FS_HD double nu(double T) const {
        double x = clog(2.34e-1, 1.57e2, T);
        double s = FS_F32(-32.275912575f) + FS_F32(1.45173283977f) * x + FS_F32(0.00936933121094f) * pow(x, 2.0)
                 + FS_F32(0.129397015353f) * pow(x, 3.0) + FS_F32(-0.0414865809044f) * pow(x, 4.0)
                 + FS_F32(-0.0582934303409f) * pow(x, 5.0) + FS_F32(0.0309832277826f) * pow(x, 6.0)
                 + FS_F32(-0.00542014733763f) * q7(x) + FS_F32(0.000325615321708f) * pow(x, 8.0);
        return exp(s) / x03 * ninf * t0;
    }
    FS_HD double beta(double T) const {
        const double a = 11.604505e3;
        double x = log10(fmin(T * ph0 / 1.5 * a, 5e4));
        return pow(10.0, 0.944 - 0.665 * (x - FS_F32(2.48f))) * 1e-13 * t0 / x03;
    }
    FS_HD double k_sc(double T) const {
        double x = log(fmin(16.0, fmax(5e-1, T * ph0)));
        double s = FS_F32(-21.4827864151f) + FS_F32(0.457356923276f) * x + FS_F32(-0.555439231606f) * pow(x, 2.0)
                 + FS_F32(1.27257798891f) * pow(x, 3.0) + FS_F32(-0.67840685073f) * pow(x, 4.0)
                 + FS_F32(0.10591014464f) * pow(x, 5.0);
        return exp(s) / 1.0e6 / x03 * t0;
    }
    FS_HD double k_si(double T) const {
        double x = log(fmin(16.0, fmax(5e-1, T * ph0)));
        double s = FS_F32(-43.1347385848f) + FS_F32(43.9905424566f) * x + FS_F32(-28.1169537586f) * pow(x, 2.0)
                 + FS_F32(8.28853856817f) * pow(x, 3.0) + FS_F32(-0.931626144207f) * pow(x, 4.0);
        return exp(s) / 1.0e6 / x03 * t0;
    }
};

// the fit evaluator of a configuration (host only)
FitEval fs_fit_eval(const fs_constants &k);
