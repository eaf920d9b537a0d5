// Shared device/host helpers for the getm_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "getm_gb300.h"

// Physical constants of python/src/wrapper.F90:11-13 (module pygetm).
#define GETM_RHO0 1025.0
#define GETM_KAPPA 0.4
#define GETM_G 9.81

// Grid handle: index extent plus device pointers to the static metrics that
// the reference reads from its type_getm_grid (src/domain/domain.F90:85-140)
// inside advection_uv_calculate / c_momentum_diffusion.
struct getm_grid {
    int imin, imax, jmin, jmax, kmin, kmax;  // Fortran 1-based interior bounds
    int halox, haloy;
    int nx_, ny_;                            // full extents incl. halos
    const int* mask;
    const double* dx;
    const double* dy;
    const double* idx;
    const double* idy;
    const double* iarea;
    const double* area;
    // float copies of the metrics for the mixed form, built on first use by
    // getm_grid_f32_metrics (device memory owned by the handle)
    float* dx_f;
    float* dy_f;
    float* idx_f;
    float* idy_f;
    float* iarea_f;
};

// Build the float metric copies of a grid if they do not exist yet (one
// cudaMalloc per array and a conversion kernel on `stream`, synchronised with
// the whole device before and after); returns a GETM_* status.  The first
// mixed-form call on a grid makes them, so that call must precede any stream
// capture.
int getm_grid_f32_metrics(getm_grid* g, cudaStream_t stream);

// Launch-shape knob of the calling host thread (GETM_TUNE_*; getm_tune_set).
int getm_tune(int knob);

// Host-side count of kernel launches issued by this library (one increment
// per launch site executed); read with getm_launch_count().
extern "C" unsigned long long getm_launch_counter_add(void);

#define GETM_CHECK_LAUNCH()                                     \
    do {                                                        \
        getm_launch_counter_add();                              \
        cudaError_t e_ = cudaGetLastError();                    \
        if (e_ != cudaSuccess) return GETM_ERR_CUDA;            \
    } while (0)

static inline unsigned int getm_div_up(long long a, long long b) { return (unsigned int)((a + b - 1) / b); }

// Thread-per-column kernels launched over a flattened range of rows: thread
// t of a 1D grid takes column (j0 + t / width, t % width) of rows j0 ..
// j0 + nrows - 1 (consecutive threads, consecutive points, rows back to back,
// so every block is full whatever the row length); false past the last
// column.  Launch getm_div_up(width * nrows, threads) blocks.
__device__ __forceinline__ bool getm_flat_column(int width, int j0, int nrows, int& i, int& j)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)width * nrows) return false;
    const int r = (int)(t / width);
    j = j0 + r;
    i = (int)(t - (long long)r * width);
    return true;
}

// ---------------------------------------------------------------------------
// double <-> float conversions on the integer pipe.  GB300 runs FP64
// instructions, conversions between double and float included, at a small
// fraction of its FP32/integer rate, so the mixed form's kernels convert the
// FP64 thickness fields by rearranging IEEE-754 bit fields instead.
// getm_f2d: exact float -> double for normal numbers and zeros.
// getm_d2f_approx: double -> float with the mantissa truncated to 23 bits
// (relative error below 2^-23; used only where a float approximation of a
// thickness is needed, e.g. as a divisor of an increment), for doubles in the
// normal float range.  Values outside those ranges take the hardware path.
// ---------------------------------------------------------------------------
// Out-of-line fallbacks: keeping the hardware conversions out of the common
// path stops the compiler from issuing them predicated on every call.
static __device__ __noinline__ double getm_f2d_hw(float x) { return (double)x; }
static __device__ __noinline__ float getm_d2f_hw(double x) { return (float)x; }

__device__ __forceinline__ double getm_f2d(float x)
{
    const unsigned int b = __float_as_uint(x);
    const unsigned int e = (b >> 23) & 0xffu;
    if (e == 0u) {
        if ((b & 0x7fffffu) == 0u)  // signed zero
            return __longlong_as_double((long long)((unsigned long long)(b >> 31) << 63));
        return getm_f2d_hw(x);  // subnormal
    }
    if (e == 0xffu) return getm_f2d_hw(x);  // inf, nan
    const unsigned long long s = (unsigned long long)(b >> 31) << 63;
    const unsigned long long m = (unsigned long long)(b & 0x7fffffu) << 29;
    const unsigned long long de = (unsigned long long)(e + (1023u - 127u)) << 52;
    return __longlong_as_double((long long)(s | de | m));
}

__device__ __forceinline__ float getm_d2f_approx(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ffu) - 1023 + 127;
    if (e <= 0 || e >= 0xff) {
        if ((b << 1) == 0ull) return __uint_as_float((unsigned int)(b >> 63) << 31);  // signed zero
        return getm_d2f_hw(x);  // outside the normal float range
    }
    const unsigned int s = (unsigned int)(b >> 63) << 31;
    const unsigned int m = (unsigned int)((b >> 29) & 0x7fffffu);
    return __uint_as_float(s | ((unsigned int)e << 23) | m);
}

// Increment-form helpers for a field stored as S (float, or double for the
// FP64 storage of the mixed form's 2D momentum and tracers): a value or a
// difference of neighbouring values (formed in S) narrowed to the float
// arithmetic of the increments, and a float increment added in S.
template <typename S>
__device__ __forceinline__ float inc_f(S x)
{
    if constexpr (std::is_same<S, double>::value) return getm_d2f_approx(x);
    else return x;
}

template <typename S>
__device__ __forceinline__ S inc_add(S x, float dx)
{
    if constexpr (std::is_same<S, double>::value) return x + getm_f2d(dx);
    else return x + dx;
}

// A value of the storage type T widened to double: float on the integer pipe
// (getm_f2d, exact), double as it is.
template <typename T>
__device__ __forceinline__ double getm_widen(T x)
{
    if constexpr (std::is_same<T, float>::value) return getm_f2d(x);
    else return x;
}

// x * 2^-n (n = 1, 2) on the integer pipe: exact, and bitwise the FP64
// multiply's result, for normal x whose product stays normal (the exponent
// field decreases by n); zeros, subnormals, infinities and NaNs take the FP64
// multiply out of line (so that it is not issued predicated on every call).
static __device__ __noinline__ double getm_scale_hw(double x, double f) { return x * f; }

template <int N>
__device__ __forceinline__ double getm_pow2_scale_down(double x)
{
    static_assert(N == 1 || N == 2, "halving or quartering");
    const long long b = __double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e > N && e < 0x7ff) return __longlong_as_double(b - ((long long)N << 52));
    return getm_scale_hw(x, N == 1 ? 0.5 : 0.25);
}

__device__ __forceinline__ double getm_half(double x) { return getm_pow2_scale_down<1>(x); }
__device__ __forceinline__ double getm_quarter(double x) { return getm_pow2_scale_down<2>(x); }

// The rest x - getm_f2d(getm_d2f_approx(x)) as a float, on the integer pipe:
// the truncated head keeps the top 24 significant bits of x, so the rest is
// the low 29 bits of the mantissa at the scale of x's last bit (rounded to 24
// bits by the conversion).  |x| below 2^-74 or beyond the float range: the
// FP64 subtraction.
__device__ __forceinline__ float getm_d2f_rest(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ffu) - 1023;
    if (e < -74 || e > 127) return getm_d2f_approx(x - getm_f2d(getm_d2f_approx(x)));
    const float r = __uint2float_rn((unsigned int)b & 0x1fffffffu) * __uint_as_float((unsigned int)(e + 75) << 23);
    return (b >> 63) ? -r : r;
}

// Comparisons of doubles on the integer pipe, for the mixed form: GB300
// issues an FP64 instruction (compare, min and max included) at a small
// fraction of the integer rate, and these give the same values.
// getm_dkey maps a double to a signed 64-bit key whose order is the numeric
// order of all non-NaN doubles (-0 orders below +0): the magnitude bits of
// a negative value are inverted.
__device__ __forceinline__ long long getm_dkey(double x)
{
    const long long b = __double_as_longlong(x);
    return b ^ (long long)((unsigned long long)(b >> 63) >> 1);
}

__device__ __forceinline__ bool getm_isnan_i(double x)
{
    return ((unsigned long long)__double_as_longlong(x) << 1) > (0x7ff0000000000000ull << 1);
}

// fmax / fmin semantics (a NaN operand yields the other one)
__device__ __forceinline__ double getm_fmax_i(double a, double b)
{
    if (getm_isnan_i(a)) return b;
    if (getm_isnan_i(b)) return a;
    return getm_dkey(a) >= getm_dkey(b) ? a : b;
}

__device__ __forceinline__ double getm_fmin_i(double a, double b)
{
    if (getm_isnan_i(a)) return b;
    if (getm_isnan_i(b)) return a;
    return getm_dkey(a) <= getm_dkey(b) ? a : b;
}

// x > 0.0 (false for NaN)
__device__ __forceinline__ bool getm_positive_i(double x)
{
    const long long b = __double_as_longlong(x);
    return b > 0 && b <= 0x7ff0000000000000ll;
}

// num / den in FP64 to about 2^-46 relative (not correctly rounded), for the
// mixed form: the float reciprocal of den refined by one Newton-Raphson step
// (q0 = num r, q = q0 + r (num - q0 den)), three FP64 instructions instead of
// a correctly rounded division.  den zero, not finite or outside the normal
// float range: the correctly rounded division.
__device__ __forceinline__ double getm_div_refined(double num, double den)
{
    const float df = getm_d2f_approx(den);
    const float adf = fabsf(df);
    if (!(adf > 1e-30f && adf < 1e30f)) return num / den;
    const double r = getm_f2d(__frcp_rn(df));
    const double q0 = num * r;
    return fma(fma(-q0, den, num), r, q0);
}

// True for the mixed form's float bulk type.  Its update kernels use the
// increment form x_new = x_old + dx, with dx formed from small differences,
// so a field that does not change is reproduced exactly and float32 rounding
// scales with the change rather than with the field; the FP64 form keeps the
// reference's evaluation order operation by operation.
template <typename T>
constexpr bool getm_increment_form = std::is_same<T, float>::value;

// ---------------------------------------------------------------------------
// TVD limiter (src/operators/advection_schemes/limiters.h:1-44).  T is the
// arithmetic type: double for the FP64 form, float for the mixed form.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T getm_limiter(int scheme, T ratio, T cfl)
{
    T limiter;
    switch (scheme) {
    case GETM_SCHEME_HSIMT: {
        T kappa = T(1) - cfl;
        T x = T(0.25) * (kappa - T(1.0) / T(3.0) / kappa);
        limiter = (T(0.5) + x) + (T(0.5) - x) * ratio;
        limiter = fmax(T(0), limiter);
        limiter = fmin(fmin(T(2) * ratio, limiter), T(2));
        break;
    }
    case GETM_SCHEME_MUSCL:
        limiter = fmin(fmin(T(2) * ratio, T(0.5) * (T(1) + ratio)), T(2));
        break;
    case GETM_SCHEME_P2_PDM: {
        T x = T(1.0) / T(6.0) * (T(1) - T(2) * cfl);
        limiter = (T(0.5) + x) + (T(0.5) - x) * ratio;
        limiter = fmin(fmin(T(2) * ratio / (cfl + T(1.e-10)), limiter), T(2) / (T(1) - cfl));
        break;
    }
    case GETM_SCHEME_SPLMAX13:
        limiter = fmin(fmin(T(2) * ratio, T(1.0) / T(3.0) * fmax(T(1) + T(2) * ratio, T(2) + ratio)), T(2));
        break;
    case GETM_SCHEME_SUPERBEE:
        limiter = fmax(fmin(T(2) * ratio, T(1)), fmin(ratio, T(2)));
        break;
    default:
        limiter = T(0);
        break;
    }
    return limiter;
}

// One TVD face value: given upstream-upstream, upstream and downstream values
// and the face Courant number, return the limited face value
// (advection.F90.template:82-88, 344-350).
template <typename T>
__device__ __forceinline__ T getm_tvd_face(int scheme, T fuu, T fu, T fd, T cfl)
{
    T deltaf = fd - fu;
    T deltafu = fu - fuu;
    if (deltaf * deltafu > T(0)) {
        T ratio = deltafu / deltaf;
        T limiter = getm_limiter<T>(scheme, ratio, cfl);
        fu = fu + T(0.5) * limiter * (T(1) - cfl) * deltaf;
    }
    return fu;
}

// The limited part of the TVD face value, face - fu (0 where the limiter is
// inactive), from the differences deltaf = fd - fu and deltafu = fu - fuu:
// the same arithmetic as getm_tvd_face without the final sum, so the
// increment form can work with deviations from cell values.
template <typename T>
__device__ __forceinline__ T getm_tvd_dev_d(int scheme, T deltaf, T deltafu, T cfl)
{
    if (deltaf * deltafu > T(0)) {
        T ratio = deltafu / deltaf;
        T limiter = getm_limiter<T>(scheme, ratio, cfl);
        return T(0.5) * limiter * (T(1) - cfl) * deltaf;
    }
    return T(0);
}

template <typename T>
__device__ __forceinline__ T getm_tvd_dev(int scheme, T fuu, T fu, T fd, T cfl)
{
    return getm_tvd_dev_d<T>(scheme, fd - fu, fu - fuu, cfl);
}

// Float form of the limited deviation without a division per field.  For
// deltaf and deltafu of the same sign s, phi(r) deltaf with r = deltafu /
// deltaf equals s phi_a(a, b), a = |deltaf|, b = |deltafu|, where phi_a is
// the limiter's expression with r replaced by b and every constant term
// multiplied by a (all five limiters are piecewise linear in r).  The terms
// that depend only on the Courant number are formed once per face
// (getm_tvd_face_f) and shared by every field advected through the face.
struct TvdFaceF {
    int scheme;
    float half1mc;     // 0.5 (1 - cfl)
    float lin0, lin1;  // HSIMT, P2_PDM: phi = lin0 + lin1 r
    float rcoef, cap;  // P2_PDM: 2 / (cfl + 1e-10), 2 / (1 - cfl)
};

__device__ __forceinline__ TvdFaceF getm_tvd_face_f(int scheme, float cfl)
{
    TvdFaceF f;
    f.scheme = scheme;
    f.half1mc = 0.5f * (1.f - cfl);
    f.lin0 = f.lin1 = 0.f;
    f.rcoef = f.cap = 2.f;
    if (scheme == GETM_SCHEME_HSIMT) {
        const float kappa = 1.f - cfl;
        const float x = 0.25f * (kappa - 1.f / 3.f / kappa);
        f.lin0 = 0.5f + x;
        f.lin1 = 0.5f - x;
    } else if (scheme == GETM_SCHEME_P2_PDM) {
        const float x = 1.f / 6.f * (1.f - 2.f * cfl);
        f.lin0 = 0.5f + x;
        f.lin1 = 0.5f - x;
        f.rcoef = 2.f / (cfl + 1.e-10f);
        f.cap = 2.f / (1.f - cfl);
    }
    return f;
}

__device__ __forceinline__ float getm_tvd_dev_f(const TvdFaceF& tf, float deltaf, float deltafu)
{
    if (!(deltaf * deltafu > 0.f)) return 0.f;
    const float a = fabsf(deltaf), b = fabsf(deltafu);
    float pa;
    switch (tf.scheme) {
    case GETM_SCHEME_HSIMT: pa = fminf(fminf(2.f * b, fmaxf(0.f, tf.lin0 * a + tf.lin1 * b)), 2.f * a); break;
    case GETM_SCHEME_MUSCL: pa = fminf(fminf(2.f * b, 0.5f * (a + b)), 2.f * a); break;
    case GETM_SCHEME_P2_PDM: pa = fminf(fminf(tf.rcoef * b, tf.lin0 * a + tf.lin1 * b), tf.cap * a); break;
    case GETM_SCHEME_SPLMAX13: pa = fminf(fminf(2.f * b, 1.f / 3.f * fmaxf(a + 2.f * b, 2.f * a + b)), 2.f * a); break;
    case GETM_SCHEME_SUPERBEE: pa = fmaxf(fminf(2.f * b, a), fminf(b, 2.f * a)); break;
    default: pa = 0.f; break;
    }
    return tf.half1mc * copysignf(pa, deltaf);
}

__device__ __forceinline__ bool getm_flux_point(int m) { return m == 1 || m == 2; }

// u*u + v*v rounded after each operation (no contraction into an FMA), so
// every kernel that forms a speed from two components gets the same bits.
__device__ __forceinline__ double getm_speed2(double u, double v) { return __dadd_rn(__dmul_rn(u, u), __dmul_rn(v, v)); }
__device__ __forceinline__ float getm_speed2(float u, float v) { return __fadd_rn(__fmul_rn(u, u), __fmul_rn(v, v)); }
