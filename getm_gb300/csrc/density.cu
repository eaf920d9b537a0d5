// Device equation of state for the baroclinic step (sm_103a).
//
// pygetm computes in-situ density with TEOS-10 through pygsw
// (python/pygetm/density.py:62-95, simulation.py:1178-1184), an external
// package that the reference does not vendor.  This library uses the
// simplified nonlinear equation of state of Roquet et al. (2015, J. Phys.
// Oceanogr. 45, "Defining a simplified yet realistic equation of state for
// seawater"), with depth (m) standing in for pressure (dbar) as the
// reference's layer-centre depth does, and returns buoyancy
// b = -g/rho0 (rho - rho0) exactly as simulation.py:1184 forms it.
#include "getm_common.cuh"

#define SEOS_RHO0 1026.0
#define SEOS_A0 1.6550e-1
#define SEOS_B0 7.6554e-1
#define SEOS_LAMBDA1 5.9520e-2
#define SEOS_LAMBDA2 5.4914e-4
#define SEOS_MU1 1.4970e-4
#define SEOS_MU2 1.1090e-5
#define SEOS_NU 2.4341e-3

__device__ __forceinline__ double seos_rho(double S, double T, double z)
{
    double Ta = T - 10.0;
    double Sa = S - 35.0;
    return SEOS_RHO0 - SEOS_A0 * (1.0 + 0.5 * SEOS_LAMBDA1 * Ta + SEOS_MU1 * z) * Ta
           + SEOS_B0 * (1.0 - 0.5 * SEOS_LAMBDA2 * Sa - SEOS_MU2 * z) * Sa - SEOS_NU * Ta * Sa;
}

// R: type of salinity and temperature.  Density and buoyancy are evaluated
// and stored in FP64 in both forms: rho - rho0 cancels three significant
// digits, and the internal pressure gradient is a small difference of large
// column integrals of buoyancy.
template <typename R>
__global__ void density_kernel(long long n, const R* S, const R* T, const double* p, double* rho, double* buoy)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    double r = seos_rho((double)S[q], (double)T[q], p[q]);
    if (rho) rho[q] = r;
    if (buoy) buoy[q] = (-GETM_G / GETM_RHO0) * (r - GETM_RHO0);
}

extern "C" int getm_density_buoyancy(int n, const double* salt, const double* temp, const double* p,
                                     double* rho, double* buoy, cudaStream_t stream)
{
    if (n < 0 || (n > 0 && (!salt || !temp || !p || (!rho && !buoy)))) return GETM_ERR_ARG;
    if (n == 0) return GETM_OK;
    density_kernel<double><<<getm_div_up(n, 256), 256, 0, stream>>>(n, salt, temp, p, rho, buoy);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_density_buoyancy_f32(int n, const float* salt, const float* temp, const double* p,
                                         double* rho, double* buoy, cudaStream_t stream)
{
    if (n < 0 || (n > 0 && (!salt || !temp || !p || (!rho && !buoy)))) return GETM_ERR_ARG;
    if (n == 0) return GETM_OK;
    density_kernel<float><<<getm_div_up(n, 256), 256, 0, stream>>>(n, salt, temp, p, rho, buoy);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}
