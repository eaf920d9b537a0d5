// Domain totals of volume and tracer content with compensated summation.
//
// Reference: python/pygetm/simulation.py:1409-1444 (Simulation.totals):
//   total_volume = sum over unmasked T points of D * area
//   tracer total = sum over unmasked T points and layers of c * area * hn
// reduced by Array.global_sum (python/pygetm/core.py:820-839), a plain numpy
// sum over the interior.  Here every partial sum is a double-double
// (hi, lo) pair built with error-free two-sums (Knuth's TwoSum, Dekker's
// FastTwoSum), so the result is the correctly rounded sum to within a few
// units in the last place whatever the field's size; the reduction order is
// fixed (no floating-point atomics), so results are bitwise reproducible.
// These are the mixed form's FP64 budget sums: float32 tracers are widened
// to double before the product.

#include "getm_common.cuh"

namespace {

struct DD {
    double hi, lo;
};

__device__ __forceinline__ DD two_sum(double a, double b)
{
    double s = a + b;
    double bb = s - a;
    double e = (a - (s - bb)) + (b - bb);
    return {s, e};
}

__device__ __forceinline__ DD dd_add(DD a, double b)
{
    DD s = two_sum(a.hi, b);
    s.lo += a.lo;
    double hi = s.hi + s.lo;  // FastTwoSum renormalisation (|s.hi| >= |s.lo|)
    return {hi, s.lo - (hi - s.hi)};
}

__device__ __forceinline__ DD dd_merge(DD a, DD b)
{
    DD s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    double hi = s.hi + s.lo;
    return {hi, s.lo - (hi - s.hi)};
}

constexpr int TOT_THREADS = 256;

template <typename T>
struct TotArgs {
    int nx_, ny_, nz, ilo, ihi, jlo, jhi;
    long long plane;
    const int* mask;
    const double* area;
    const double* D;
    const double* hn;
    int ntracer;
    const T* tr[GETM_MAX_TOTALS];
    double* partial;  // [nfields][gridDim.x][2]
};

// Block-wide fixed-order tree reduction of one DD per thread.
__device__ DD block_reduce(DD v)
{
    __shared__ double shi[TOT_THREADS], slo[TOT_THREADS];
    shi[threadIdx.x] = v.hi;
    slo[threadIdx.x] = v.lo;
    __syncthreads();
    for (int s = TOT_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            DD r = dd_merge({shi[threadIdx.x], slo[threadIdx.x]}, {shi[threadIdx.x + s], slo[threadIdx.x + s]});
            shi[threadIdx.x] = r.hi;
            slo[threadIdx.x] = r.lo;
        }
        __syncthreads();
    }
    DD r = {shi[0], slo[0]};
    __syncthreads();
    return r;
}

// blockIdx.y = field (0: volume, 1 + t: tracer t); grid-stride over the
// interior columns.
template <typename T>
__global__ void __launch_bounds__(TOT_THREADS) totals_partial_kernel(TotArgs<T> a)
{
    const int field = blockIdx.y;
    const int ni = a.ihi - a.ilo + 1;
    const long long ncol = (long long)ni * (a.jhi - a.jlo + 1);
    DD acc = {0.0, 0.0};
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < ncol;
         q += (long long)gridDim.x * blockDim.x) {
        const int j = a.jlo + (int)(q / ni);
        const int i = a.ilo + (int)(q - (q / ni) * ni);
        const long long c = (long long)j * a.nx_ + i;
        if (a.mask[c] == 0) continue;
        const double ar = a.area[c];
        if (field == 0) {
            acc = dd_add(acc, a.D[c] * ar);
        } else {
            const T* f = a.tr[field - 1];
            for (int k = 0; k < a.nz; k++) {
                const long long p = c + k * a.plane;
                acc = dd_add(acc, ((double)f[p] * ar) * a.hn[p]);
            }
        }
    }
    DD r = block_reduce(acc);
    if (threadIdx.x == 0) {
        double* out = a.partial + 2 * ((long long)field * gridDim.x + blockIdx.x);
        out[0] = r.hi;
        out[1] = r.lo;
    }
}

// One block per field: reduce the per-block partials in a fixed order.
__global__ void __launch_bounds__(TOT_THREADS) totals_final_kernel(const double* partial, int nblk, double* out)
{
    const int field = blockIdx.x;
    const double* p = partial + 2LL * field * nblk;
    DD acc = {0.0, 0.0};
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) acc = dd_merge(acc, {p[2 * b], p[2 * b + 1]});
    DD r = block_reduce(acc);
    if (threadIdx.x == 0) out[field] = r.hi + r.lo;
}

template <typename T>
int totals_impl(int nx_, int ny_, int nz, int halox, int haloy, int nx, int ny, const int* mask,
                const double* area, const double* D, const double* hn, int ntracer, const T* const* tracers,
                double* work, double* out, cudaStream_t stream)
{
    if (nx_ < 1 || ny_ < 1 || nz < 1 || nx < 1 || ny < 1 || halox < 0 || haloy < 0) return GETM_ERR_ARG;
    if (halox + nx > nx_ || haloy + ny > ny_) return GETM_ERR_ARG;
    if (!mask || !area || !D || !work || !out) return GETM_ERR_ARG;
    if (ntracer < 0 || ntracer > GETM_MAX_TOTALS || (ntracer > 0 && (!hn || !tracers))) return GETM_ERR_ARG;
    TotArgs<T> a;
    a.nx_ = nx_; a.ny_ = ny_; a.nz = nz;
    a.ilo = halox; a.ihi = halox + nx - 1; a.jlo = haloy; a.jhi = haloy + ny - 1;
    a.plane = (long long)nx_ * ny_;
    a.mask = mask; a.area = area; a.D = D; a.hn = hn; a.ntracer = ntracer;
    for (int t = 0; t < GETM_MAX_TOTALS; t++) a.tr[t] = t < ntracer ? tracers[t] : nullptr;
    for (int t = 0; t < ntracer; t++)
        if (!a.tr[t]) return GETM_ERR_ARG;
    a.partial = work;
    long long ncol = (long long)nx * ny;
    int nblk = (int)((ncol + TOT_THREADS - 1) / TOT_THREADS);
    if (nblk > GETM_TOTALS_BLOCKS) nblk = GETM_TOTALS_BLOCKS;
    dim3 grid(nblk, 1 + ntracer);
    totals_partial_kernel<T><<<grid, TOT_THREADS, 0, stream>>>(a);
    GETM_CHECK_LAUNCH();
    totals_final_kernel<<<1 + ntracer, TOT_THREADS, 0, stream>>>(work, nblk, out);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

}  // namespace

extern "C" int getm_domain_totals(int nx_, int ny_, int nz, int halox, int haloy, int nx, int ny,
                                  const int* mask, const double* area, const double* D, const double* hn,
                                  int ntracer, const double* const* tracers, double* work, double* out,
                                  cudaStream_t stream)
{
    return totals_impl<double>(nx_, ny_, nz, halox, haloy, nx, ny, mask, area, D, hn, ntracer, tracers, work,
                               out, stream);
}

extern "C" int getm_domain_totals_f32(int nx_, int ny_, int nz, int halox, int haloy, int nx, int ny,
                                      const int* mask, const double* area, const double* D, const double* hn,
                                      int ntracer, const float* const* tracers, double* work, double* out,
                                      cudaStream_t stream)
{
    return totals_impl<float>(nx_, ny_, nz, halox, haloy, nx, ny, mask, area, D, hn, ntracer, tracers, work,
                              out, stream);
}
