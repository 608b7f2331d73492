// fs_sg.cuh -- get_Flux (ptcl_props.F90:142-165) for a general charge q,
// mobility and diffusion coefficient, for the faces that have no shared-
// exponential fast path (the dielectric wall, where the energy flux takes
// get_mut/get_Dt rather than 5/3 mue, 5/3 De).  Near a = 0 the Bernoulli form
// replaces the closed form, whose 1 - exp(-a) cancels, as on every other face.
#pragma once
#include <cuda_runtime.h>

__device__ __forceinline__ double fs_sg_flux(double q, double E, double dh, double mu, double D, double nl,
                                             double nr) {
    const double tol = 9.9999999600419720025e-13;   // REAL(4) 1e-12
    const double v = q * mu * E;
    const double arg = v * dh / D;
    if (fabs(q * E) < tol) return D * (nl - nr) / dh;
    if (fabs(arg) < 1e-2) {
        const double a2 = arg * arg;
        return D * ((nl - nr) + 0.5 * arg * (nl + nr) + a2 * (1.0 / 12.0 - a2 / 720.0) * (nl - nr)) / dh;
    }
    if (arg > 0) {
        const double ex = exp(fmax(-arg, -100.0));
        return v * (nl - nr * ex) / (1.0 - ex);
    }
    const double ex = exp(fmax(arg, -100.0));
    return v * (nr - nl * ex) / (1.0 - ex);
}
