// Momentum kernels of python/src/momentum.F90 and c_momentum_diffusion of
// python/src/wrapper.F90:275-393, for sm_103a.
//
// Elementwise work maps one thread to one output point with warps along i;
// the stencils that the reference evaluates as "flux array, then divergence"
// recompute the two face fluxes of each point in registers instead of
// writing a flux array (no intermediate traffic).  Column recursions
// (w_momentum_3d) use one thread per column.
#include "split2d_ops.cuh"

#include <type_traits>

#define EW_THREADS 256

// momentum.F90:12-77
__global__ void horizontal_diffusion_kernel(int nx_, int ny_, int ilo, int ihi, int jlo, int jhi,
                                            const int* umask, const int* vmask, const double* idxu,
                                            const double* dyu, const double* idyv, const double* dxv,
                                            const double* Ah_u, const double* Ah_v, const int* tmask,
                                            const double* iA, double dt, const double* f, double* df)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i < ilo || i > ihi || j < jlo || j > jhi) return;
    long long p = (long long)j * nx_ + i;
    if (tmask[p] != 1) return;
    long long w = p - 1, s = p - nx_;
    double ufe = (umask[p] == 1) ? Ah_u[p] * (f[p + 1] - f[p]) * idxu[p] * dyu[p] : 0.0;
    double ufw = (umask[w] == 1) ? Ah_u[w] * (f[w + 1] - f[w]) * idxu[w] * dyu[w] : 0.0;
    double vfn = (vmask[p] == 1) ? Ah_v[p] * (f[p + nx_] - f[p]) * idyv[p] * dxv[p] : 0.0;
    double vfs = (vmask[s] == 1) ? Ah_v[s] * (f[s + nx_] - f[s]) * idyv[s] * dxv[s] : 0.0;
    df[p] = dt * (ufe - ufw + vfn - vfs) * iA[p];
}

extern "C" int getm_horizontal_diffusion(int imin, int imax, int jmin, int jmax, int halox, int haloy,
                                         const int* umask, const int* vmask, const double* idxu,
                                         const double* dyu, const double* idyv, const double* dxv,
                                         const double* Ah_u, const double* Ah_v, const int* tmask,
                                         const double* iA, double dt, const double* f, double* out,
                                         cudaStream_t stream)
{
    if (imax < imin || jmax < jmin || halox < 1 || haloy < 1) return GETM_ERR_ARG;
    if (!umask || !vmask || !idxu || !dyu || !idyv || !dxv || !Ah_u || !Ah_v || !tmask || !iA || !f || !out)
        return GETM_ERR_ARG;
    int nx_ = imax - imin + 1 + 2 * halox, ny_ = jmax - jmin + 1 + 2 * haloy;
    dim3 grid(getm_div_up(nx_, 128), ny_);
    horizontal_diffusion_kernel<<<grid, 128, 0, stream>>>(nx_, ny_, halox, halox + imax - imin, haloy, haloy + jmax - jmin,
                                                          umask, vmask, idxu, dyu, idyv, dxv, Ah_u, Ah_v, tmask, iA, dt, f, out);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// momentum.F90:79-101.  C: arithmetic type of the drag coefficient (double:
// the reference arithmetic; float: the mixed form, which evaluates the
// logarithm and square roots of this coefficient in float and stores the
// result in double).
template <typename C>
__global__ void bottom_friction_kernel(int n, const int* mask, const double* u, const double* v,
                                       const double* D, double* z0b, const double* z0b_min,
                                       double avmmol, double* ru, int iterate)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n || mask[p] != 1) return;
    C uu = (C)u[p], vv = (C)v[p], DD = (C)D[p];
    C z0 = (C)z0b[p];
    C sqrtcd = C(GETM_KAPPA) / log(C(1) + C(0.5) * DD / z0);
    if (iterate != 0) {
        z0 = fmin(DD, (C)z0b_min[p] + C(0.1) * (C)avmmol / fmax((C)avmmol, sqrtcd * sqrt(getm_speed2(uu, vv))));
        z0b[p] = z0;
        sqrtcd = C(GETM_KAPPA) / log(C(1) + C(0.5) * DD / z0);
    }
    ru[p] = sqrtcd * sqrtcd * sqrt(getm_speed2(uu, vv));
}

template <typename C>
static int bottom_friction_impl(int nx, int ny, const int* mask, const double* u, const double* v, const double* D,
                                double* z0b, const double* z0b_in, double avmmol, double* ru, int iterate,
                                cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || !mask || !u || !v || !D || !z0b || !ru || (iterate && !z0b_in)) return GETM_ERR_ARG;
    int n = nx * ny;
    bottom_friction_kernel<C><<<getm_div_up(n, EW_THREADS), EW_THREADS, 0, stream>>>(n, mask, u, v, D, z0b, z0b_in, avmmol, ru, iterate);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_bottom_friction(int nx, int ny, const int* mask, const double* u, const double* v,
                                    const double* D, double* z0b, const double* z0b_in, double avmmol,
                                    double* ru, int iterate, cudaStream_t stream)
{
    return bottom_friction_impl<double>(nx, ny, mask, u, v, D, z0b, z0b_in, avmmol, ru, iterate, stream);
}

extern "C" int getm_bottom_friction_mixed(int nx, int ny, const int* mask, const double* u, const double* v,
                                          const double* D, double* z0b, const double* z0b_in, double avmmol,
                                          double* ru, int iterate, cudaStream_t stream)
{
    return bottom_friction_impl<float>(nx, ny, mask, u, v, D, z0b, z0b_in, avmmol, ru, iterate, stream);
}

// momentum.F90:103-145: rows haloy..ny-haloy-1, every i, every k (mask unused).
// T: type of the 3D tendency fields and of ea2/ea4; the internal pressure
// gradient idp is double in both forms; the FP64 form sums in FP64, the
// mixed form (float sources) in float.
template <typename T>
__global__ void collect_sources_kernel(int nx, int ny, int nz, int haloy, const double* __restrict__ alpha,
                                       const double* __restrict__ ho, const double* __restrict__ hn, const double* __restrict__ dp,
                                       const T* __restrict__ cor, const T* __restrict__ adv, const T* __restrict__ diff,
                                       const double* __restrict__ idp, const double* __restrict__ taus, const double* __restrict__ rr,
                                       double dt, T* __restrict__ ea2, T* __restrict__ ea4)
{
    // one thread per cell: grid (flattened columns, level)
    int i, j;
    if (!getm_flat_column(nx, haloy, ny - 2 * haloy, i, j)) return;
    const int k = blockIdx.y;
    long long plane = (long long)nx * ny;
    long long p = (long long)j * nx + i;
    const long long q = p + k * plane;
    const double al = alpha[p], dpp = dp[p];
    const double rho0i = 1.0 / GETM_RHO0;
    if constexpr (getm_increment_form<T>) {
        // mixed form: the sources are stored in float, so they are summed
        // in float (each term to float precision)
        const float alf = getm_d2f_approx(al), dtf = (float)dt;
        const float gdp = (float)(-0.5 * GETM_G) * getm_d2f_approx(dpp);
        float e = dtf * (gdp * (getm_d2f_approx(ho[q]) + getm_d2f_approx(hn[q])) +
                         alf * (cor[q] + adv[q] + diff[q] + getm_d2f_approx(idp[q])));
        if (k == nz - 1) e = e + dtf * alf * getm_d2f_approx(taus[p]) * (float)rho0i;
        ea4[q] = e;
        if (k == 0) ea2[p] = -dtf * getm_d2f_approx(rr[p]);
        return;
    }
    double e = dt * (-0.5 * (ho[q] + hn[q]) * GETM_G * dpp
                     + al * ((double)cor[q] + (double)adv[q] + (double)diff[q] + idp[q]));
    if (k == nz - 1) e = e + dt * al * taus[p] * rho0i;
    ea4[q] = (T)e;
    if (k == 0) ea2[p] = (T)(-dt * rr[p]);
}

template <typename T>
static int collect_impl(int nx, int ny, int nz, int haloy, const double* alpha, const double* ho, const double* hn,
                        const double* dp, const T* cor, const T* adv, const T* diff, const double* idp,
                        const double* taus, const double* rr, double dt, T* ea2, T* ea4, cudaStream_t stream)
{
    if (nx < 1 || ny <= 2 * haloy || nz < 1 || !alpha || !ho || !hn || !dp || !cor || !adv || !diff || !idp || !taus || !rr || !ea2 || !ea4)
        return GETM_ERR_ARG;
    const dim3 grid(getm_div_up((long long)nx * (ny - 2 * haloy), 128), nz);
    collect_sources_kernel<T><<<grid, 128, 0, stream>>>(nx, ny, nz, haloy, alpha, ho, hn, dp, cor, adv, diff, idp, taus, rr, dt, ea2, ea4);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_collect_3d_momentum_sources(int nx, int ny, int nz, int halox, int haloy,
                                                const int* mask, const double* alpha, const double* ho,
                                                const double* hn, const double* dp, const double* cor,
                                                const double* adv, const double* diff, const double* idp,
                                                const double* taus, const double* rr, double dt,
                                                double* ea2, double* ea4, cudaStream_t stream)
{
    (void)mask; (void)halox;
    return collect_impl<double>(nx, ny, nz, haloy, alpha, ho, hn, dp, cor, adv, diff, idp, taus, rr, dt, ea2, ea4, stream);
}

extern "C" int getm_collect_3d_momentum_sources_f32(int nx, int ny, int nz, int halox, int haloy,
                                                    const int* mask, const double* alpha, const double* ho,
                                                    const double* hn, const double* dp, const float* cor,
                                                    const float* adv, const float* diff, const double* idp,
                                                    const double* taus, const double* rr, double dt,
                                                    float* ea2, float* ea4, cudaStream_t stream)
{
    (void)mask; (void)halox;
    return collect_impl<float>(nx, ny, nz, haloy, alpha, ho, hn, dp, cor, adv, diff, idp, taus, rr, dt, ea2, ea4, stream);
}

// momentum.F90:147-189
__global__ void advance_2d_transport_kernel(int nx, int ny, int halox, int haloy, Transport2DArgs a, double dt)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i < halox || i >= nx - halox || j < haloy || j >= ny - haloy) return;
    transport_2d_point(a, dt, (long long)j * nx + i);
}

extern "C" int getm_advance_2d_transport(int nx, int ny, int halox, int haloy, const int* mask,
                                         const double* alpha, const double* D, const double* dp,
                                         const double* taus, const double* cor, const double* adv,
                                         const double* diff, const double* damp, const double* SA,
                                         const double* SB, const double* SD, const double* SF,
                                         const double* r, double dt, double* U, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || !mask || !alpha || !D || !dp || !taus || !cor || !adv || !diff || !damp || !SA || !SB || !SD || !SF || !r || !U)
        return GETM_ERR_ARG;
    dim3 grid(getm_div_up(nx, 128), ny);
    Transport2DArgs a{mask, alpha, D, dp, taus, cor, adv, diff, damp, SA, SB, SD, SF, r, U};
    advance_2d_transport_kernel<<<grid, 128, 0, stream>>>(nx, ny, halox, haloy, a, dt);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// momentum.F90:191-216: thread per column; the recursion runs in FP64 for
// both forms (T: type of pk, qk and w).
template <typename T>
__global__ void w_momentum_3d_kernel(int nx, int ny, int nz, int ilo, int ihi, int jlo, int jhi,
                                     const int* __restrict__ mask, const double* __restrict__ dyu, const double* __restrict__ dxv,
                                     const double* __restrict__ iarea, const double* __restrict__ ho, const double* __restrict__ hn,
                                     const T* __restrict__ pk, const T* __restrict__ qk, double dt, T* __restrict__ w)
{
    int i, j;
    if (!getm_flat_column(nx, jlo, jhi - jlo + 1, i, j) || i < ilo || i > ihi) return;
    long long p = (long long)j * nx + i;
    if (mask[p] != 1) return;
    long long plane = (long long)nx * ny;
    const double idt = 1.0 / dt;
    const double dyE = dyu[p], dyW = dyu[p - 1], dxN = dxv[p], dxS = dxv[p - nx], ia = iarea[p];
    if constexpr (std::is_same<T, double>::value) {
        double wk = (double)w[p];
        for (int k = 1; k <= nz - 1; k++) {
            long long q = p + (k - 1) * plane;
            wk = wk - (hn[q] - ho[q]) * idt
                 - ((double)pk[q] * dyE - (double)pk[q - 1] * dyW + (double)qk[q] * dxN - (double)qk[q - nx] * dxS) * ia;
            w[p + k * plane] = (T)wk;
        }
    } else {
        // mixed form: the layer's increment in float (the thickness change
        // differenced in FP64 first), accumulated up the column in FP64
        const float idtf = (float)idt;
        const float dyEf = getm_d2f_approx(dyE), dyWf = getm_d2f_approx(dyW);
        const float dxNf = getm_d2f_approx(dxN), dxSf = getm_d2f_approx(dxS), iaf = getm_d2f_approx(ia);
        double wk = getm_f2d(w[p]);
        for (int k = 1; k <= nz - 1; k++) {
            long long q = p + (k - 1) * plane;
            const float inc = getm_d2f_approx(hn[q] - ho[q]) * idtf +
                              (pk[q] * dyEf - pk[q - 1] * dyWf + qk[q] * dxNf - qk[q - nx] * dxSf) * iaf;
            wk = wk - getm_f2d(inc);
            w[p + k * plane] = getm_d2f_approx(wk);
        }
    }
}

template <typename T>
static int w_momentum_impl(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax, const int* mask,
                           const double* dyu, const double* dxv, const double* iarea, const double* ho,
                           const double* hn, const T* pk, const T* qk, double dt, T* w, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || imin < 2 || jmin < 2 || imax > nx || jmax > ny || jmax < jmin) return GETM_ERR_ARG;
    if (!mask || !dyu || !dxv || !iarea || !ho || !hn || !pk || !qk || !w) return GETM_ERR_ARG;
    const unsigned grid = getm_div_up((long long)nx * (jmax - jmin + 1), 128);
    w_momentum_3d_kernel<T><<<grid, 128, 0, stream>>>(nx, ny, nz, imin - 1, imax - 1, jmin - 1, jmax - 1, mask, dyu, dxv, iarea, ho, hn, pk, qk, dt, w);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_w_momentum_3d(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                                  const int* mask, const double* dyu, const double* dxv,
                                  const double* iarea, const double* ho, const double* hn,
                                  const double* pk, const double* qk, double dt, double* w,
                                  cudaStream_t stream)
{
    return w_momentum_impl<double>(nx, ny, nz, imin, imax, jmin, jmax, mask, dyu, dxv, iarea, ho, hn, pk, qk, dt, w, stream);
}

extern "C" int getm_w_momentum_3d_f32(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                                      const int* mask, const double* dyu, const double* dxv,
                                      const double* iarea, const double* ho, const double* hn,
                                      const float* pk, const float* qk, double dt, float* w,
                                      cudaStream_t stream)
{
    return w_momentum_impl<float>(nx, ny, nz, imin, imax, jmin, jmax, mask, dyu, dxv, iarea, ho, hn, pk, qk, dt, w, stream);
}

// momentum.F90:218-241 (T: type of uk, vk, SS and of the arithmetic)
template <typename T>
__global__ void shear_frequency_kernel(int nx, int ny, int nz, int ilo, int ihi, int jlo, int jhi,
                                       const int* __restrict__ mask, const double* __restrict__ hu, const double* __restrict__ hv,
                                       const T* __restrict__ uk, const T* __restrict__ vk, T* __restrict__ SS)
{
    int i, j;
    const int k = blockIdx.y + 1;  // Fortran interface k = 1..nz-1
    if (!getm_flat_column(nx, jlo, jhi - jlo + 1, i, j) || i < ilo || i > ihi) return;
    long long p = (long long)j * nx + i;
    if (mask[p] <= 0) return;
    long long plane = (long long)nx * ny;
    long long a = p + (k - 1) * plane, b = p + k * plane;
    // thicknesses in T (float: narrowed on the integer pipe)
    auto h = [](double x) -> T {
        if constexpr (std::is_same<T, double>::value) return x;
        else return getm_d2f_approx(x);
    };
    T t1 = (uk[b] - uk[a]) / (T(0.5) * (h(hu[b]) + h(hu[a])));
    T t2 = (uk[b - 1] - uk[a - 1]) / (T(0.5) * (h(hu[b - 1]) + h(hu[a - 1])));
    T t3 = (vk[b] - vk[a]) / (T(0.5) * (h(hv[b]) + h(hv[a])));
    T t4 = (vk[b - nx] - vk[a - nx]) / (T(0.5) * (h(hv[b - nx]) + h(hv[a - nx])));
    SS[b] = T(0.5) * (t1 * t1 + t2 * t2 + t3 * t3 + t4 * t4);
}

template <typename T>
static int shear_impl(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax, const int* mask,
                      const double* hu, const double* hv, const T* uk, const T* vk, T* SS, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || imin < 2 || jmin < 2 || imax > nx || jmax > ny || jmax < jmin) return GETM_ERR_ARG;
    if (!mask || !hu || !hv || !uk || !vk || !SS) return GETM_ERR_ARG;
    if (nz < 2) return GETM_OK;
    dim3 grid(getm_div_up((long long)nx * (jmax - jmin + 1), 128), nz - 1);
    shear_frequency_kernel<T><<<grid, 128, 0, stream>>>(nx, ny, nz, imin - 1, imax - 1, jmin - 1, jmax - 1, mask, hu, hv, uk, vk, SS);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// c_shear_frequency2 (momentum.F90:244-268): the squared shear frequency
// weighted by the viscosity at the four neighbouring velocity points,
// normalised by the viscosity of the T point; interfaces k = 1..nz-1 of the
// interior T points with mask > 0.  The same expression and operation order.
template <typename T>
__global__ void shear_frequency2_kernel(int nx, int ny, int nz, int ilo, int ihi, int jlo, int jhi,
                                        const int* __restrict__ mask, const double* __restrict__ h,
                                        const double* __restrict__ hu, const double* __restrict__ hv,
                                        const T* __restrict__ uk, const T* __restrict__ vk,
                                        const T* __restrict__ num, T* __restrict__ SS)
{
    int i, j;
    const int k = blockIdx.y + 1;  // Fortran interface k = 1..nz-1
    if (!getm_flat_column(nx, jlo, jhi - jlo + 1, i, j) || i < ilo || i > ihi) return;
    const long long p = (long long)j * nx + i;
    if (mask[p] <= 0) return;
    const long long plane = (long long)nx * ny;
    const long long a = p + (k - 1) * plane, b = p + k * plane;  // layers Fortran k, k+1
    const long long q = p + k * plane;                            // interface k
    auto c = [](double x) -> T {
        if constexpr (std::is_same<T, double>::value) return x;
        else return getm_d2f_approx(x);
    };
    const T due = uk[b] - uk[a], duw = uk[b - 1] - uk[a - 1];
    const T dvn = vk[b] - vk[a], dvs = vk[b - nx] - vk[a - nx];
    const T s = due * due / (c(hu[b]) + c(hu[a])) * (num[q] + num[q + 1])
                + duw * duw / (c(hu[b - 1]) + c(hu[a - 1])) * (num[q - 1] + num[q])
                + dvn * dvn / (c(hv[b]) + c(hv[a])) * (num[q] + num[q + nx])
                + dvs * dvs / (c(hv[b - nx]) + c(hv[a - nx])) * (num[q - nx] + num[q]);
    SS[q] = T(0.5) * s / (T(0.5) * (c(h[a]) + c(h[b]))) / num[q];
}

template <typename T>
static int shear2_impl(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax, const int* mask,
                       const double* h, const double* hu, const double* hv, const T* uk, const T* vk, const T* num,
                       T* SS, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || imin < 2 || jmin < 2 || imax >= nx || jmax >= ny || jmax < jmin)
        return GETM_ERR_ARG;
    if (!mask || !h || !hu || !hv || !uk || !vk || !num || !SS) return GETM_ERR_ARG;
    if (nz < 2) return GETM_OK;
    dim3 grid(getm_div_up((long long)nx * (jmax - jmin + 1), 128), nz - 1);
    shear_frequency2_kernel<T><<<grid, 128, 0, stream>>>(nx, ny, nz, imin - 1, imax - 1, jmin - 1, jmax - 1, mask, h,
                                                          hu, hv, uk, vk, num, SS);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_shear_frequency2(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax, const int* mask,
                                     const double* h, const double* hu, const double* hv, const double* uk,
                                     const double* vk, const double* num, double* SS, cudaStream_t stream)
{
    return shear2_impl<double>(nx, ny, nz, imin, imax, jmin, jmax, mask, h, hu, hv, uk, vk, num, SS, stream);
}

extern "C" int getm_shear_frequency2_f32(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                                         const int* mask, const double* h, const double* hu, const double* hv,
                                         const float* uk, const float* vk, const float* num, float* SS,
                                         cudaStream_t stream)
{
    return shear2_impl<float>(nx, ny, nz, imin, imax, jmin, jmax, mask, h, hu, hv, uk, vk, num, SS, stream);
}

extern "C" int getm_shear_frequency(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                                    const int* mask, const double* hu, const double* hv, const double* uk,
                                    const double* vk, double* SS, cudaStream_t stream)
{
    return shear_impl<double>(nx, ny, nz, imin, imax, jmin, jmax, mask, hu, hv, uk, vk, SS, stream);
}

extern "C" int getm_shear_frequency_f32(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                                        const int* mask, const double* hu, const double* hv, const float* uk,
                                        const float* vk, float* SS, cudaStream_t stream)
{
    return shear_impl<float>(nx, ny, nz, imin, imax, jmin, jmax, mask, hu, hv, uk, vk, SS, stream);
}

// momentum.F90:270-284
__global__ void surface_shear_velocity_kernel(int nx, int ilo, int ihi, int jlo, int jhi, const int* mask,
                                              const double* taux, const double* tauy, double* ustar)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y + jlo;
    if (i < ilo || i > ihi || j > jhi) return;
    long long p = (long long)j * nx + i;
    if (mask[p] > 0) {
        const double rho0i = 1.0 / GETM_RHO0;
        ustar[p] = pow(taux[p] * taux[p] + tauy[p] * tauy[p], 0.25) * sqrt(rho0i);
    }
}

extern "C" int getm_surface_shear_velocity(int nx, int ny, int imin, int imax, int jmin, int jmax,
                                           const int* mask, const double* tausx, const double* tausy,
                                           double* ustar2_s, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || imin < 1 || jmin < 1 || imax > nx || jmax > ny || jmax < jmin) return GETM_ERR_ARG;
    if (!mask || !tausx || !tausy || !ustar2_s) return GETM_ERR_ARG;
    dim3 grid(getm_div_up(nx, 128), jmax - jmin + 1);
    surface_shear_velocity_kernel<<<grid, 128, 0, stream>>>(nx, imin - 1, imax - 1, jmin - 1, jmax - 1, mask, tausx, tausy, ustar2_s);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// momentum.F90:286-321.  The two stress components are stored on their
// rows and recomputed in registers where the shear velocity needs a
// neighbour's value (same product, same result).
__global__ void bottom_shear_velocity_kernel(int nx, int ny, int ilo, int ihi, int jlo, int jhi,
                                             const int* mask, const double* uk_bot, const double* vk_bot,
                                             const double* rru, const double* rrv, double* ustar2_x,
                                             double* ustar2_y, double* ustar)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= nx || j >= ny) return;
    long long p = (long long)j * nx + i;
    if (j >= jlo && j <= jhi) ustar2_x[p] = -uk_bot[p] * rru[p];
    if (j >= jlo - 1 && j <= jhi) ustar2_y[p] = -vk_bot[p] * rrv[p];
    if (i >= ilo && i <= ihi && j >= jlo && j <= jhi && mask[p] == 1) {
        double a = -uk_bot[p - 1] * rru[p - 1];
        double b = -uk_bot[p] * rru[p];
        double c = -vk_bot[p - nx] * rrv[p - nx];
        double d = -vk_bot[p] * rrv[p];
        ustar[p] = pow(0.5 * (a * a + b * b + c * c + d * d), 0.25);
    }
}

extern "C" int getm_bottom_shear_velocity(int nx, int ny, int imin, int imax, int jmin, int jmax,
                                          const int* mask, const int* umask, const int* vmask,
                                          const double* uk_bot, const double* vk_bot, const double* rru,
                                          const double* rrv, double* taubx, double* tauby,
                                          double* ustar2_b, cudaStream_t stream)
{
    (void)umask; (void)vmask;
    if (nx < 1 || ny < 1 || imin < 2 || jmin < 2 || imax > nx || jmax > ny || jmax < jmin) return GETM_ERR_ARG;
    if (!mask || !uk_bot || !vk_bot || !rru || !rrv || !taubx || !tauby || !ustar2_b) return GETM_ERR_ARG;
    dim3 grid(getm_div_up(nx, 128), ny);
    bottom_shear_velocity_kernel<<<grid, 128, 0, stream>>>(nx, ny, imin - 1, imax - 1, jmin - 1, jmax - 1, mask, uk_bot, vk_bot, rru, rrv, taubx, tauby, ustar2_b);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// Momentum.advance_3d_transport after the vertical diffusion
// (python/pygetm/momentum.py:1199-1210): tp3d = vel hn, dev = (sum_k tp3d -
// tp2d) / D, tp3d -= dev hn, as one sweep per column (the sum in FP64 in
// both forms).  FP64 form (T double): the same roundings as the separate
// array operations (products and differences not contracted); the sum runs
// bottom to top.  Mixed form (T float): the products in float from the
// thickness narrowed on the integer pipe.
template <typename T>
__global__ void transport_3d_finish_kernel(long long plane, int nz, const T* __restrict__ vel, const double* __restrict__ hn,
                                           const double* __restrict__ tp2d, const double* __restrict__ D, T* __restrict__ tp3d, double* __restrict__ dev)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= plane) return;
    double s = 0.0;
    for (int k = 0; k < nz; k++) {
        const long long q = p + k * plane;
        T x;
        if constexpr (std::is_same<T, double>::value) x = __dmul_rn(vel[q], hn[q]);
        else x = vel[q] * getm_d2f_approx(hn[q]);
        tp3d[q] = x;
        s = s + getm_widen(x);
    }
    const double d = (s - tp2d[p]) / D[p];
    dev[p] = d;
    for (int k = 0; k < nz; k++) {
        const long long q = p + k * plane;
        if constexpr (std::is_same<T, double>::value) tp3d[q] = __dsub_rn(tp3d[q], __dmul_rn(d, hn[q]));
        else tp3d[q] = tp3d[q] - getm_d2f_approx(d) * getm_d2f_approx(hn[q]);
    }
}

// Column sums of up to four 3D fields into 2D FP64 fields (the slow terms of
// momentum.py:989-1012 and simulation.py:1186-1192): dst = sum_k src
// (- dst when subtract is set), summed bottom to top in FP64; NULL pairs are
// skipped.
template <typename T>
__global__ void column_sums_kernel(long long plane, int nz, int subtract, const T* __restrict__ a3,
                                   double* __restrict__ a2, const T* __restrict__ b3, double* __restrict__ b2,
                                   const T* __restrict__ c3, double* __restrict__ c2, const T* __restrict__ d3,
                                   double* __restrict__ d2)
{
    // one field per grid row (blockIdx.y), one column per thread
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    const T* src = f == 0 ? a3 : f == 1 ? b3 : f == 2 ? c3 : d3;
    double* dst = f == 0 ? a2 : f == 1 ? b2 : f == 2 ? c2 : d2;
    if (p >= plane || !src) return;
    double s = 0.0;
    for (int k = 0; k < nz; k++) s = s + getm_widen(src[p + k * plane]);
    dst[p] = subtract ? s - dst[p] : s;
}

template <typename T>
static int column_sums_impl(int nx, int ny, int nz, int subtract, const T* a3, double* a2, const T* b3, double* b2,
                            const T* c3, double* c2, const T* d3, double* d2, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1) return GETM_ERR_ARG;
    if (!a3 != !a2 || !b3 != !b2 || !c3 != !c2 || !d3 != !d2) return GETM_ERR_ARG;
    const long long plane = (long long)nx * ny;
    column_sums_kernel<T><<<dim3(getm_div_up(plane, 128), 4), 128, 0, stream>>>(plane, nz, subtract, a3, a2, b3, b2,
                                                                                 c3, c2, d3, d2);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_column_sums(int nx, int ny, int nz, int subtract, const double* a3, double* a2,
                                const double* b3, double* b2, const double* c3, double* c2, const double* d3,
                                double* d2, cudaStream_t stream)
{
    return column_sums_impl<double>(nx, ny, nz, subtract, a3, a2, b3, b2, c3, c2, d3, d2, stream);
}

extern "C" int getm_column_sums_f32(int nx, int ny, int nz, int subtract, const float* a3, double* a2,
                                    const float* b3, double* b2, const float* c3, double* c2, const float* d3,
                                    double* d2, cudaStream_t stream)
{
    return column_sums_impl<float>(nx, ny, nz, subtract, a3, a2, b3, b2, c3, c2, d3, d2, stream);
}

// Momentum.update_diagnostics (momentum.py:909-910): uk = pk / hn, vk = qk /
// hn over n points (mixed form: in float).
template <typename T>
__global__ void velocities_3d_kernel(long long n, const T* pk, const double* hnu, const T* qk, const double* hnv,
                                     T* uk, T* vk, long long plane = 0, double* ubot = nullptr,
                                     double* vbot = nullptr)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    T u, v;
    if constexpr (std::is_same<T, double>::value) {
        u = pk[q] / hnu[q];
        v = qk[q] / hnv[q];
    } else {
        u = pk[q] / getm_d2f_approx(hnu[q]);
        v = qk[q] / getm_d2f_approx(hnv[q]);
    }
    uk[q] = u;
    vk[q] = v;
    if (ubot && q < plane) {  // the bottom layer widened to FP64 (exact)
        ubot[q] = getm_widen(u);
        vbot[q] = getm_widen(v);
    }
}

template <typename T>
static int transport_3d_finish_impl(int nx, int ny, int nz, const T* vel, const double* hn, const double* tp2d,
                                    const double* D, T* tp3d, double* dev, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || !vel || !hn || !tp2d || !D || !tp3d || !dev) return GETM_ERR_ARG;
    const long long plane = (long long)nx * ny;
    transport_3d_finish_kernel<T><<<getm_div_up(plane, 128), 128, 0, stream>>>(plane, nz, vel, hn, tp2d, D, tp3d, dev);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_transport_3d_finish(int nx, int ny, int nz, const double* vel, const double* hn,
                                        const double* tp2d, const double* D, double* tp3d, double* dev,
                                        cudaStream_t stream)
{
    return transport_3d_finish_impl<double>(nx, ny, nz, vel, hn, tp2d, D, tp3d, dev, stream);
}

extern "C" int getm_transport_3d_finish_f32(int nx, int ny, int nz, const float* vel, const double* hn,
                                            const double* tp2d, const double* D, float* tp3d, double* dev,
                                            cudaStream_t stream)
{
    return transport_3d_finish_impl<float>(nx, ny, nz, vel, hn, tp2d, D, tp3d, dev, stream);
}

template <typename T>
static int velocities_3d_impl(long long n, const T* pk, const double* hnu, const T* qk, const double* hnv, T* uk,
                              T* vk, cudaStream_t stream)
{
    if (n < 0 || (n > 0 && (!pk || !hnu || !qk || !hnv || !uk || !vk))) return GETM_ERR_ARG;
    if (n == 0) return GETM_OK;
    velocities_3d_kernel<T><<<getm_div_up(n, 256), 256, 0, stream>>>(n, pk, hnu, qk, hnv, uk, vk);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_velocities_3d(long long n, const double* pk, const double* hnu, const double* qk,
                                  const double* hnv, double* uk, double* vk, cudaStream_t stream)
{
    return velocities_3d_impl<double>(n, pk, hnu, qk, hnv, uk, vk, stream);
}

extern "C" int getm_velocities_3d_f32(long long n, const float* pk, const double* hnu, const float* qk,
                                      const double* hnv, float* uk, float* vk, cudaStream_t stream)
{
    return velocities_3d_impl<float>(n, pk, hnu, qk, hnv, uk, vk, stream);
}

extern "C" int getm_velocities_3d_bottom_f32(long long n, long long plane, const float* pk, const double* hnu,
                                             const float* qk, const double* hnv, float* uk, float* vk, double* ubot,
                                             double* vbot, cudaStream_t stream)
{
    if (n < 0 || plane < 0 || plane > n || (n > 0 && (!pk || !hnu || !qk || !hnv || !uk || !vk || !ubot || !vbot)))
        return GETM_ERR_ARG;
    if (n == 0) return GETM_OK;
    velocities_3d_kernel<float><<<getm_div_up(n, 256), 256, 0, stream>>>(n, pk, hnu, qk, hnv, uk, vk, plane, ubot,
                                                                          vbot);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// Momentum.advance (momentum.py:790-793): the mean transports of the
// substeps, Ui = U_cum / split_factor (as a product with the reciprocal,
// like the reference's numpy expression), then U_cum = 0.
__global__ void mean_transports_kernel(long long n, double* Ucum, double* Vcum, double scale, double* Ui, double* Vi)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    Ui[q] = Ucum[q] * scale;
    Vi[q] = Vcum[q] * scale;
    Ucum[q] = 0.0;
    Vcum[q] = 0.0;
}

extern "C" int getm_mean_transports(long long n, double* Ucum, double* Vcum, double scale, double* Ui, double* Vi,
                                    cudaStream_t stream)
{
    if (n < 0 || (n > 0 && (!Ucum || !Vcum || !Ui || !Vi))) return GETM_ERR_ARG;
    if (n == 0) return GETM_OK;
    mean_transports_kernel<<<getm_div_up(n, 256), 256, 0, stream>>>(n, Ucum, Vcum, scale, Ui, Vi);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// Momentum.update_diagnostics (momentum.py:1003-1015): the slow bottom
// friction SxF = ustar2_bx + ru u1 (SyF likewise), product and sum rounded
// separately as in the reference's numpy expression (no contraction).
__global__ void slow_friction_kernel(long long n, const double* ustar2x, const double* ru, const double* u1,
                                     double* SxF, const double* ustar2y, const double* rv, const double* v1,
                                     double* SyF)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    SxF[q] = __dadd_rn(ustar2x[q], __dmul_rn(ru[q], u1[q]));
    SyF[q] = __dadd_rn(ustar2y[q], __dmul_rn(rv[q], v1[q]));
}

extern "C" int getm_slow_friction(long long n, const double* ustar2x, const double* ru, const double* u1,
                                  double* SxF, const double* ustar2y, const double* rv, const double* v1, double* SyF,
                                  cudaStream_t stream)
{
    if (n < 0 || (n > 0 && (!ustar2x || !ru || !u1 || !SxF || !ustar2y || !rv || !v1 || !SyF))) return GETM_ERR_ARG;
    if (n == 0) return GETM_OK;
    slow_friction_kernel<<<getm_div_up(n, 256), 256, 0, stream>>>(n, ustar2x, ru, u1, SxF, ustar2y, rv, v1, SyF);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// momentum.F90:323-340: rows jmin..jmax, every i (T: type of un and Uo)
template <typename T>
__global__ void reconstruct_kernel(int nx, int ny, int nz, int jlo, int jhi, T* un, const double* hn,
                                   const T* Uo, double idt)
{
    long long plane = (long long)nx * ny;
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= plane * nz) return;
    int j = (int)((p % plane) / nx);
    if (j < jlo || j > jhi) return;
    reconstruct_point<T>(un, hn, Uo, idt, p);
}

template <typename T>
static int reconstruct_impl(int nx, int ny, int nz, int jmin, int jmax, T* un, const double* hn, const T* Uo,
                            double timestep, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || jmin < 1 || jmax > ny || !un || !hn || !Uo) return GETM_ERR_ARG;
    long long n = (long long)nx * ny * nz;
    reconstruct_kernel<T><<<getm_div_up(n, EW_THREADS), EW_THREADS, 0, stream>>>(nx, ny, nz, jmin - 1, jmax - 1, un, hn, Uo, 1.0 / timestep);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_reconstruct_transport_change(int nx, int ny, int nz, int imin, int imax, int jmin,
                                                 int jmax, double* un, const double* hn, const double* Uo,
                                                 double timestep, cudaStream_t stream)
{
    (void)imin; (void)imax;
    return reconstruct_impl<double>(nx, ny, nz, jmin, jmax, un, hn, Uo, timestep, stream);
}

extern "C" int getm_reconstruct_transport_change_f32(int nx, int ny, int nz, int imin, int imax, int jmin,
                                                     int jmax, float* un, const double* hn, const float* Uo,
                                                     double timestep, cudaStream_t stream)
{
    (void)imin; (void)imax;
    return reconstruct_impl<float>(nx, ny, nz, jmin, jmax, un, hn, Uo, timestep, stream);
}

// wrapper.F90:275-393 (one layer per blockIdx.z).  All six grids share the
// extent of the U grid (python/pygetm/domain.py:699-725).
struct MomDiffArgs {
    int nx, ny, ilo, ihi, jlo, jhi;
    const int *umask, *vmask, *uumask, *uvmask, *vumask, *vvmask;
    const double *uiarea, *viarea, *uudy, *uuidx, *uvdx, *uvidx, *uvidy, *vudy, *vuidx, *vuidy, *vvdx, *vvidy;
    const double *huu, *huv, *hvu, *hvv, *u, *v;
    double Am0;
    double *diffu, *diffv;
};

__global__ void momentum_diffusion_kernel(MomDiffArgs a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    int k = blockIdx.z;
    if (i < a.ilo || i > a.ihi || j < a.jlo || j > a.jhi) return;
    const long long nx = a.nx;
    long long p = (long long)j * nx + i;
    long long off = (long long)k * nx * a.ny;
    const double* u = a.u + off;
    const double* v = a.v + off;
    const double Am0 = a.Am0;
#define FUU(q) ((a.uumask[q] != 0) ? 2.0 * Am0 * a.uudy[q] * a.huu[off + (q)] * (u[(q) + 1] - u[q]) * a.uuidx[q] : 0.0)
#define FUV(q) ((a.uvmask[q] != 0) ? Am0 * a.uvdx[q] * a.huv[off + (q)] * ((u[(q) + nx] - u[q]) * a.uvidy[q] + (v[(q) + 1] - v[q]) * a.uvidx[q]) : 0.0)
#define FVU(q) ((a.vumask[q] != 0) ? Am0 * a.vudy[q] * a.hvu[off + (q)] * ((u[(q) + nx] - u[q]) * a.vuidy[q] + (v[(q) + 1] - v[q]) * a.vuidx[q]) : 0.0)
#define FVV(q) ((a.vvmask[q] != 0) ? 2.0 * Am0 * a.vvdx[q] * a.hvv[off + (q)] * (v[(q) + nx] - v[q]) * a.vvidy[q] : 0.0)
    // diffu: :323-356
    double du = 0.0;
    int um = a.umask[p];
    if (um == 1) du = (FUU(p) - FUU(p - 1)) * a.uiarea[p];
    if (um == 1 || um == 2) du = du + (FUV(p) - FUV(p - nx)) * a.uiarea[p];
    a.diffu[off + p] = du;
    // diffv: :358-391
    double dv = 0.0;
    if (a.vmask[p] == 1) {
        dv = (FVU(p) - FVU(p - 1)) * a.viarea[p];
        dv = dv + (FVV(p) - FVV(p - nx)) * a.viarea[p];
    }
    a.diffv[off + p] = dv;
#undef FUU
#undef FUV
#undef FVU
#undef FVV
}

extern "C" int getm_momentum_diffusion(getm_grid* UG, getm_grid* VG, getm_grid* UUG, getm_grid* UVG,
                                       getm_grid* VUG, getm_grid* VVG, int nk, const double* huu,
                                       const double* huv, const double* hvu, const double* hvv,
                                       const double* u, const double* v, double Am0, double* diffu,
                                       double* diffv, cudaStream_t stream)
{
    if (!UG || !VG || !UUG || !UVG || !VUG || !VVG || nk < 1) return GETM_ERR_ARG;
    if (!huu || !huv || !hvu || !hvv || !u || !v || !diffu || !diffv) return GETM_ERR_ARG;
    MomDiffArgs a;
    a.nx = UG->nx_; a.ny = UG->ny_;
    a.ilo = UG->halox; a.ihi = UG->halox + UG->imax - UG->imin;
    a.jlo = UG->haloy; a.jhi = UG->haloy + UG->jmax - UG->jmin;
    a.umask = UG->mask; a.vmask = VG->mask; a.uumask = UUG->mask; a.uvmask = UVG->mask;
    a.vumask = VUG->mask; a.vvmask = VVG->mask;
    a.uiarea = UG->iarea; a.viarea = VG->iarea;
    a.uudy = UUG->dy; a.uuidx = UUG->idx;
    a.uvdx = UVG->dx; a.uvidx = UVG->idx; a.uvidy = UVG->idy;
    a.vudy = VUG->dy; a.vuidx = VUG->idx; a.vuidy = VUG->idy;
    a.vvdx = VVG->dx; a.vvidy = VVG->idy;
    a.huu = huu; a.huv = huv; a.hvu = hvu; a.hvv = hvv; a.u = u; a.v = v; a.Am0 = Am0;
    a.diffu = diffu; a.diffv = diffv;
    if (!a.umask || !a.vmask || !a.uumask || !a.uvmask || !a.vumask || !a.vvmask || !a.uiarea || !a.viarea ||
        !a.uudy || !a.uuidx || !a.uvdx || !a.uvidx || !a.uvidy || !a.vudy || !a.vuidx || !a.vuidy || !a.vvdx || !a.vvidy)
        return GETM_ERR_ARG;
    dim3 grid(getm_div_up(a.nx, 128), a.ny, nk);
    momentum_diffusion_kernel<<<grid, 128, 0, stream>>>(a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}
