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
#include <type_traits>

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

// ---------------------------------------------------------------------------
// Double-float arithmetic (a value as the unevaluated sum hi + lo of two
// floats, about 48 significant bits): Dekker's and Knuth's error-free
// transformations (T. J. Dekker, "A floating-point technique for extending
// the available precision", Numer. Math. 18, 1971; D. E. Knuth, TAOCP vol. 2,
// 4.2.2), the product's error from a fused multiply-add.  Every operation is
// an explicitly rounded intrinsic, so the compiler neither contracts nor
// reorders them.
// ---------------------------------------------------------------------------
struct DF {
    float hi, lo;
};

// s + e with |s| >= |e| (or s == 0), renormalised
__device__ __forceinline__ DF df_fast_sum(float s, float e)
{
    const float h = __fadd_rn(s, e);
    return DF{h, __fsub_rn(e, __fsub_rn(h, s))};
}

__device__ __forceinline__ DF df_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ DF df_add(DF x, DF y)
{
    const DF s = df_two_sum(x.hi, y.hi);
    return df_fast_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}

__device__ __forceinline__ DF df_mul(DF x, DF y)
{
    const float p = __fmul_rn(x.hi, y.hi);
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, e));
    return df_fast_sum(p, e);
}

// a double constant split into its float head and the float of the rest
struct DFConst {
    float hi, lo;
    __host__ __device__ constexpr DFConst(double c) : hi((float)c), lo((float)(c - (double)(float)c)) {}
};

__device__ __forceinline__ DF df_of(DFConst c) { return DF{c.hi, c.lo}; }

// The anomaly rho - rho0 of seos_rho in double-float from float S, T (exact
// inputs) and the FP64 depth (split exactly into a truncated float head and
// the float of the rest: one FP64 subtraction).  The anomaly is formed
// without the constant rho0, so the cancellation of rho - rho0 that the FP64
// form suffers does not occur: its error is some 1e-14 of the anomaly.
__device__ __forceinline__ DF seos_anomaly_df(float S, float T, double z)
{
    constexpr DFConst A0(SEOS_A0), B0(SEOS_B0), L1(0.5 * SEOS_LAMBDA1), L2(0.5 * SEOS_LAMBDA2);
    constexpr DFConst M1(SEOS_MU1), M2(SEOS_MU2), NU(SEOS_NU);
    const float zh = getm_d2f_approx(z);
    const DF zd{zh, getm_d2f_approx(z - getm_f2d(zh))};
    const DF Ta = df_two_sum(T, -10.f);
    const DF Sa = df_two_sum(S, -35.f);
    const DF one{1.f, 0.f};
    // (1 + l1/2 Ta + m1 z) Ta, (1 - l2/2 Sa - m2 z) Sa
    const DF u = df_add(one, df_add(df_mul(df_of(L1), Ta), df_mul(df_of(M1), zd)));
    DF v = df_add(df_mul(df_of(L2), Sa), df_mul(df_of(M2), zd));
    v = df_add(one, DF{-v.hi, -v.lo});
    const DF tA = df_mul(df_of(A0), df_mul(u, Ta));
    const DF tB = df_mul(df_of(B0), df_mul(v, Sa));
    const DF tN = df_mul(df_of(NU), df_mul(Ta, Sa));
    return df_add(df_add(DF{-tA.hi, -tA.lo}, tB), DF{-tN.hi, -tN.lo});
}

// The same anomaly from FP64 S and T (the mixed form's FP64 tracer storage):
// each is split into a truncated float head and the float of the rest (both
// on the integer pipe), which the double-float sums take in.
__device__ __forceinline__ DF seos_anomaly_df2(double S, double T, double z)
{
    constexpr DFConst A0(SEOS_A0), B0(SEOS_B0), L1(0.5 * SEOS_LAMBDA1), L2(0.5 * SEOS_LAMBDA2);
    constexpr DFConst M1(SEOS_MU1), M2(SEOS_MU2), NU(SEOS_NU);
    const float zh = getm_d2f_approx(z), Th = getm_d2f_approx(T), Sh = getm_d2f_approx(S);
    const DF zd{zh, getm_d2f_rest(z)};
    const float Tl = getm_d2f_rest(T), Sl = getm_d2f_rest(S);
    const DF Ta = df_add(df_two_sum(Th, -10.f), DF{Tl, 0.f});
    const DF Sa = df_add(df_two_sum(Sh, -35.f), DF{Sl, 0.f});
    const DF one{1.f, 0.f};
    const DF u = df_add(one, df_add(df_mul(df_of(L1), Ta), df_mul(df_of(M1), zd)));
    DF v = df_add(df_mul(df_of(L2), Sa), df_mul(df_of(M2), zd));
    v = df_add(one, DF{-v.hi, -v.lo});
    const DF tA = df_mul(df_of(A0), df_mul(u, Ta));
    const DF tB = df_mul(df_of(B0), df_mul(v, Sa));
    const DF tN = df_mul(df_of(NU), df_mul(Ta, Sa));
    return df_add(df_add(DF{-tA.hi, -tA.lo}, tB), DF{-tN.hi, -tN.lo});
}

__global__ void density_f64s_kernel(long long n, const double* S, const double* T, const double* p, double* rho,
                                    double* buoy)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const DF a = seos_anomaly_df2(S[q], T[q], p[q]);
    if (rho) rho[q] = SEOS_RHO0 + (getm_f2d(a.hi) + getm_f2d(a.lo));
    if (buoy) {
        // -g/rho0 (anomaly + (SEOS_RHO0 - rho0)) in double-float: one FP64
        // addition to widen it
        constexpr DFConst GB(-GETM_G / GETM_RHO0);
        const DF t = df_add(a, DF{(float)(SEOS_RHO0 - GETM_RHO0), 0.f});
        const DF m = df_mul(df_of(GB), t);
        buoy[q] = getm_f2d(m.hi) + getm_f2d(m.lo);
    }
}

extern "C" int getm_density_buoyancy_f64s(int n, const double* salt, const double* temp, const double* p,
                                          double* rho, double* buoy, cudaStream_t stream)
{
    if (n < 0 || (n > 0 && (!salt || !temp || !p || (!rho && !buoy)))) return GETM_ERR_ARG;
    if (n == 0) return GETM_OK;
    density_f64s_kernel<<<getm_div_up(n, 256), 256, 0, stream>>>(n, salt, temp, p, rho, buoy);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// R: type of salinity and temperature.  Density and buoyancy are stored in
// FP64 in both forms (the internal pressure gradient is a small difference
// of large column integrals of buoyancy).  The FP64 form evaluates seos_rho
// in FP64; the mixed form (float S and T) evaluates the anomaly rho - rho0
// in double-float and widens it: five FP64 operations per point instead of
// some fifteen, and no cancellation in the buoyancy.
template <typename R>
__global__ void density_kernel(long long n, const R* S, const R* T, const double* p, double* rho, double* buoy)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    if constexpr (std::is_same<R, double>::value) {
        const double r = seos_rho(S[q], T[q], p[q]);
        if (rho) rho[q] = r;
        if (buoy) buoy[q] = (-GETM_G / GETM_RHO0) * (r - GETM_RHO0);
    } else {
        // rho - GETM_RHO0 = (SEOS_RHO0 - GETM_RHO0) + anomaly, the first
        // term an exact small integer
        const DF a = seos_anomaly_df(S[q], T[q], p[q]);
        const double ad = getm_f2d(a.hi) + getm_f2d(a.lo);
        if (rho) rho[q] = SEOS_RHO0 + ad;
        if (buoy) buoy[q] = (-GETM_G / GETM_RHO0) * (ad + (SEOS_RHO0 - GETM_RHO0));
    }
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

// ---------------------------------------------------------------------------
// Squared buoyancy frequency at the interior layer interfaces
// (Density.get_buoyancy_frequency, python/pygetm/density.py:22-60, called
// every baroclinic 3D step at simulation.py:1200-1204), for the device EOS:
// N2 = -g/rho0 (rho(S1, T1, zi) - rho(S0, T0, zi)) / dz between level k
// (below) and k + 1, both densities at the interface depth zi = (p_k +
// p_k+1)/2 (locally referenced, as TEOS-10's nsquared evaluates them at the
// mid pressure), dz = (h_k + h_k+1)/2.  The density difference is formed
// from the differences of temperature and salinity with the polynomial
// identities of the EOS, so it keeps the precision of the differences:
//   f(Ta) = (1 + l1/2 Ta + m1 z) Ta:  f(Ta1) - f(Ta0) = dT (1 + l1/2 (Ta1 + Ta0) + m1 z)
//   Ta1 Sa1 - Ta0 Sa0 = dT Sa1 + Ta0 dS.
// Interfaces 1 .. nz-1 of columns with a non-zero mask are written; the
// surface and bottom interfaces are left as they are (reference: out[1:-1]).
// R: arithmetic and the type of N2 (float in the mixed form); X: type of S
// and T (R, or double with float arithmetic for the mixed form's FP64
// tracers: the differences dT, dS are formed in FP64 and narrowed).
template <typename R, typename X = R>
__global__ void buoyancy_frequency_kernel(long long plane, int nz, const int* __restrict__ mask,
                                          const double* __restrict__ h, const double* __restrict__ p,
                                          const X* __restrict__ S, const X* __restrict__ T, R* __restrict__ NN)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;  // interface k + 1
    if (c >= plane || k >= nz - 1 || mask[c] == 0) return;
    const long long q0 = c + (long long)k * plane, q1 = q0 + plane;
    R T0, T1, S0, S1, dT, dS;
    if constexpr (std::is_same<R, X>::value) {
        T0 = T[q0]; T1 = T[q1]; S0 = S[q0]; S1 = S[q1];
        dT = T1 - T0; dS = S1 - S0;
    } else {
        const X T0x = T[q0], T1x = T[q1], S0x = S[q0], S1x = S[q1];
        T0 = getm_d2f_approx(T0x); T1 = getm_d2f_approx(T1x);
        S0 = getm_d2f_approx(S0x); S1 = getm_d2f_approx(S1x);
        dT = getm_d2f_approx(T1x - T0x); dS = getm_d2f_approx(S1x - S0x);
    }
    const R Ta0 = T0 - R(10), Ta1 = T1 - R(10), Sa0 = S0 - R(35), Sa1 = S1 - R(35);
    R zi, dz;
    if constexpr (std::is_same<R, double>::value) {
        zi = 0.5 * (p[q0] + p[q1]);
        dz = 0.5 * (h[q0] + h[q1]);
    } else {
        zi = 0.5f * (getm_d2f_approx(p[q0]) + getm_d2f_approx(p[q1]));
        dz = 0.5f * (getm_d2f_approx(h[q0]) + getm_d2f_approx(h[q1]));
    }
    const R drho = -R(SEOS_A0) * dT * (R(1) + R(0.5 * SEOS_LAMBDA1) * (Ta1 + Ta0) + R(SEOS_MU1) * zi)
                   + R(SEOS_B0) * dS * (R(1) - R(0.5 * SEOS_LAMBDA2) * (Sa1 + Sa0) - R(SEOS_MU2) * zi)
                   - R(SEOS_NU) * (dT * Sa1 + Ta0 * dS);
    NN[q1] = R(-GETM_G / GETM_RHO0) * drho / dz;
}

template <typename R>
static int buoyancy_frequency_impl(int nx, int ny, int nz, const int* mask, const double* h, const double* p,
                                   const R* S, const R* T, R* NN, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || !mask || !h || !p || !S || !T || !NN) return GETM_ERR_ARG;
    if (nz == 1) return GETM_OK;
    const long long plane = (long long)nx * ny;
    dim3 grid(getm_div_up(plane, 256), nz - 1);
    buoyancy_frequency_kernel<R><<<grid, 256, 0, stream>>>(plane, nz, mask, h, p, S, T, NN);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_buoyancy_frequency(int nx, int ny, int nz, const int* mask, const double* h, const double* p,
                                       const double* salt, const double* temp, double* NN, cudaStream_t stream)
{
    return buoyancy_frequency_impl<double>(nx, ny, nz, mask, h, p, salt, temp, NN, stream);
}

extern "C" int getm_buoyancy_frequency_f32(int nx, int ny, int nz, const int* mask, const double* h, const double* p,
                                           const float* salt, const float* temp, float* NN, cudaStream_t stream)
{
    return buoyancy_frequency_impl<float>(nx, ny, nz, mask, h, p, salt, temp, NN, stream);
}

extern "C" int getm_buoyancy_frequency_f64s(int nx, int ny, int nz, const int* mask, const double* h,
                                            const double* p, const double* salt, const double* temp, float* NN,
                                            cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || !mask || !h || !p || !salt || !temp || !NN) return GETM_ERR_ARG;
    if (nz == 1) return GETM_OK;
    const long long plane = (long long)nx * ny;
    dim3 grid(getm_div_up(plane, 256), nz - 1);
    buoyancy_frequency_kernel<float, double><<<grid, 256, 0, stream>>>(plane, nz, mask, h, p, salt, temp, NN);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}
