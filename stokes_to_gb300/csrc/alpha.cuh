// Brinkman penalty laws alpha(rho) and d alpha / d rho, shared by the 3D and 2D
// design-loop kernels.
#pragma once
#include "internal.cuh"

namespace stg {

// STG_ALPHA_REF: the reference law on s = rho^3 (fluid_topo/FluidTopoOpt3D.cpp:110-123);
// STG_ALPHA_BP: amax * 0.1 (1 - rho) / (0.1 + rho).
__device__ __forceinline__ double alpha_of(double r, const stg_alpha& L) {
    if (L.law == STG_ALPHA_REF) {
        double s = r * r * r;
        return L.alpha_os + (L.alpha_us - L.alpha_os) * s * (1 + L.q) / (s + L.q);
    }
    return L.amax * 0.1 * (1.0 - r) / (0.1 + r);
}
// d alpha / d rho including the rho^3 chain of the reference law (FluidTopoOpt3D.cpp:202-208, 273)
__device__ __forceinline__ double dalpha_of(double r, const stg_alpha& L) {
    if (L.law == STG_ALPHA_REF) {
        double s = r * r * r;
        double da = (L.alpha_us - L.alpha_os) * ((1 + L.q) / (s + L.q) - s * (1 + L.q) / ((s + L.q) * (s + L.q)));
        return da * 3.0 * (r * r);
    }
    return -L.amax * 0.1 * 1.1 / ((0.1 + r) * (0.1 + r));
}

}  // namespace stg
