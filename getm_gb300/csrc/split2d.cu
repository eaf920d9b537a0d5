// Fused sequences of the split-explicit 2D substep for sm_103a.
//
// Each 2D substep of pygetm's Simulation (python/pygetm/simulation.py
// :1033-1304, momentum.py:644-758, :1017-1148) runs some sixty small
// operations on fields of one horizontal plane (~10^5 points).  On GB300 each
// of those is a kernel launch of a few microseconds, so the substep loop is
// bound by launches rather than by memory.  The kernels below each replace a
// contiguous sequence of those operations with one launch.  Every value is a
// function of the sequence's inputs at the same or neighbouring points, so a
// point's outputs are computed by its own thread, recomputing neighbouring
// intermediates where needed; with FP64 arithmetic they evaluate the same
// expressions in the same order as the separate operations and give
// bitwise-identical results.  Points that a separate interpolation does not
// write keep their previous values here too.
//
// Layout: every field is [j][i] with the full halo-inclusive extents of its
// grid (nx_, ny_ for T, U, V and their velocity grids, nx_+1, ny_+1 for X).
#include <math.h>

#include "getm_common.cuh"

#define S2_THREADS 128

namespace {

// torch.clamp(x, min=lo): NaN propagates
__device__ __forceinline__ double clamp_min(double x, double lo) { return isnan(x) ? x : (x < lo ? lo : x); }

struct DepthArgs {
    int nx, ny;                 // T-grid extents (halos included)
    double Dmin, Dcrit, ialpha; // ialpha = 1 / (Dcrit - 2 Dmin)
    const double *z, *zo;       // elevations (T)
    const double *HT, *HU, *HV, *HX;
    const int *mT, *mU, *mV, *mX;
    double *DT, *DclipT, *workT;
    double *workU, *DU, *alphaU;
    double *workV, *DV, *alphaV;
    double *workX, *DX;         // X extents (nx+1) x (ny+1)
    double *DUU, *DVV, *DUV, *DVU;
};

constexpr int UD_BX = 32, UD_BY = 4;

// alpha (wrapper.F90:428-436) with the constant divisor as a reciprocal
__device__ __forceinline__ double alpha_of(double d, double twoDmin, double ialpha)
{
    return fmax(0.0, fmin(1.0, (d - twoDmin) * ialpha));
}

// Simulation.update_depth, 2D part (simulation.py:1498-1586 without the
// halo exchanges and mirroring of a single closed domain).  A 32 x 4 block
// covers X points (j, i) of its tile and the T, U, V points with the same
// indices; z_T_half of the tile plus a one-point halo is formed once into
// shared memory.  Copies between grids are scattered by the point that
// owns the source value (UU.D(j, i-1) = D_T_half(j, i), VV.D(j-1, i) =
// D_T_half(j, i), UV.D(j-1, i-1) = VU.D(j-1, i-1) = X.D(j, i)).
__global__ void __launch_bounds__(UD_BX * UD_BY) update_depth_2d_kernel(DepthArgs a)
{
    __shared__ double szh[UD_BY + 2][UD_BX + 2];  // z_T_half at rows j0-1.., cols i0-1..
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = blockIdx.x * UD_BX, j0 = blockIdx.y * UD_BY;
    const int i = i0 + tx, j = j0 + ty;
    const int nx = a.nx, ny = a.ny;
    for (int q = ty * UD_BX + tx; q < (UD_BY + 2) * (UD_BX + 2); q += UD_BX * UD_BY) {
        const int sj = q / (UD_BX + 2), si = q - sj * (UD_BX + 2);
        const int gj = j0 - 1 + sj, gi = i0 - 1 + si;
        double v = 0.0;
        if (gj >= 0 && gj < ny && gi >= 0 && gi < nx) {
            const long long g = (long long)gj * nx + gi;
            v = (a.zo[g] + a.z[g]) * 0.5;
        }
        szh[sj][si] = v;
    }
    __syncthreads();
    if (i > nx || j > ny) return;
    const int sj = ty + 1, si = tx + 1;  // (j, i) in the tile
    // X point (j, i): interp_xy T->X (offsets 1, 1) where it writes, else the
    // previous X._work value
    {
        const long long px = (long long)j * (nx + 1) + i;
        double zx;
        if (j >= 1 && j <= ny - 1 && i >= 1 && i <= nx - 1) {
            zx = 0.25 * (szh[sj - 1][si - 1] + szh[sj - 1][si] + szh[sj][si - 1] + szh[sj][si]);
            a.workX[px] = zx;
        } else {
            zx = a.workX[px];
        }
        double dx = a.DX[px];
        if (a.mX[px] != 0) {
            dx = fmax(a.HX[px] + zx, a.Dmin);
            a.DX[px] = dx;
        }
        if (j >= 1 && i >= 1 && j - 1 < ny && i - 1 < nx) {  // UV.D = X.D[1:, 1:]; VU.D = UV.D
            const long long q = (long long)(j - 1) * nx + (i - 1);
            a.DUV[q] = dx;
            a.DVU[q] = dx;
        }
    }
    if (i >= nx || j >= ny) return;
    const long long p = (long long)j * nx + i;
    const double zh = szh[sj][si];
    // T: elevation2depth(z, H, -1000), Dclip = clamp(D, Dmin), D_T_half
    double DT = a.DT[p];
    if (a.mT[p] != 0) DT = fmax(a.HT[p] + a.z[p], -1000.0);
    a.DT[p] = DT;
    a.DclipT[p] = clamp_min(DT, a.Dmin);
    const double dth = a.mT[p] != 0 ? fmax(a.HT[p] + zh, a.Dmin) : zh;
    a.workT[p] = dth;
    if (i >= 1) a.DUU[p - 1] = dth;   // UU.D[:, :-1] = D_T_half[:, 1:]
    if (j >= 1) a.DVV[p - nx] = dth;  // VV.D[:-1, :] = D_T_half[1:, :]
    const double twoDmin = 2 * a.Dmin;
    // U: z_U = interp_x(z_T_half, ioffset 0) for i < nx-1, else the old value
    double zu;
    if (i < nx - 1) {
        zu = 0.5 * (zh + szh[sj][si + 1]);
        a.workU[p] = zu;
    } else {
        zu = a.workU[p];
    }
    if (a.mU[p] != 0) {
        const double d = fmax(a.HU[p] + zu, a.Dmin);
        a.DU[p] = d;
        a.alphaU[p] = alpha_of(d, twoDmin, a.ialpha);
    }
    // V: z_V = interp_y(z_T_half, joffset 0) for j < ny-1
    double zv;
    if (j < ny - 1) {
        zv = 0.5 * (zh + szh[sj + 1][si]);
        a.workV[p] = zv;
    } else {
        zv = a.workV[p];
    }
    if (a.mV[p] != 0) {
        const double d = fmax(a.HV[p] + zv, a.Dmin);
        a.DV[p] = d;
        a.alphaV[p] = alpha_of(d, twoDmin, a.ialpha);
    }
}

// Momentum._transport_2d_momentum up to the advection calls
// (momentum.py:1017-1040 with Am = 0): u1 = U/DU, v1 = V/DV, the advected
// copies, and the advection velocities on the UU, UV, VU, VV grids.
// C: arithmetic of the four advection velocities (float in the mixed form).
struct VelArgs {
    int nx, ny;
    const double *U, *V, *DU, *DV, *DUU, *DUV, *DVU, *DVV;
    double *u1, *v1, *advU, *advV, *uua, *uva, *vua, *vva;
};

template <typename C>
__device__ __forceinline__ double vel_div(double num, double den)
{
    if constexpr (std::is_same<C, double>::value) return num / den;
    else return getm_f2d(getm_d2f_approx(num) / getm_d2f_approx(den));
}

template <typename C>
__global__ void __launch_bounds__(S2_THREADS) momentum_2d_velocities_kernel(VelArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= a.nx || j >= a.ny) return;
    const long long p = (long long)j * a.nx + i;
    const double u1 = a.U[p] / a.DU[p];
    const double v1 = a.V[p] / a.DV[p];
    a.u1[p] = u1; a.advU[p] = u1;
    a.v1[p] = v1; a.advV[p] = v1;
    // interp_x (ioffset 0) writes i < nx-1; elsewhere the old value is divided
    const double uu = i < a.nx - 1 ? 0.5 * (a.U[p] + a.U[p + 1]) : a.uua[p];
    const double uv = i < a.nx - 1 ? 0.5 * (a.V[p] + a.V[p + 1]) : a.uva[p];
    const double vu = j < a.ny - 1 ? 0.5 * (a.U[p] + a.U[p + a.nx]) : a.vua[p];
    const double vv = j < a.ny - 1 ? 0.5 * (a.V[p] + a.V[p + a.nx]) : a.vva[p];
    a.uua[p] = vel_div<C>(uu, a.DUU[p]);
    a.uva[p] = vel_div<C>(uv, a.DUV[p]);
    a.vua[p] = vel_div<C>(vu, a.DVU[p]);
    a.vva[p] = vel_div<C>(vv, a.DVV[p]);
}

// Momentum.bottom_friction (momentum.py:1099-1125): u1 -> V grid and v1 -> U
// grid by interp_xy, then bottom_friction on both grids (momentum.F90:79-101,
// iterate = 0).  C: arithmetic of the drag coefficient.
struct FricArgs {
    int nx, ny;
    const int *mU, *mV;
    const double *u1, *v1, *DU, *DV, *z0bU, *z0bV;
    double *workU, *workV, *ru, *rv;
};

template <typename C>
__device__ __forceinline__ double drag(double u, double v, double D, double z0)
{
    const C uu = (C)u, vv = (C)v, DD = (C)D;
    const C sqrtcd = C(GETM_KAPPA) / log(C(1) + C(0.5) * DD / (C)z0);
    return sqrtcd * sqrtcd * sqrt(getm_speed2(uu, vv));
}

template <typename C>
__global__ void __launch_bounds__(S2_THREADS) momentum_2d_friction_kernel(FricArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= a.nx || j >= a.ny) return;
    const long long p = (long long)j * a.nx + i;
    const int nx = a.nx;
    // v_U = interp_xy(v1, ioffset 0, joffset 1): written at j >= 1, i <= nx-2
    double vU = a.workU[p];
    if (j >= 1 && i <= nx - 2) {
        const long long q = p - nx;
        vU = 0.25 * (a.v1[q] + a.v1[q + 1] + a.v1[q + nx] + a.v1[q + nx + 1]);
        a.workU[p] = vU;
    }
    // u_V = interp_xy(u1, ioffset 1, joffset 0): written at i >= 1, j <= ny-2
    double uV = a.workV[p];
    if (i >= 1 && j <= a.ny - 2) {
        const long long q = p - 1;
        uV = 0.25 * (a.u1[q] + a.u1[q + 1] + a.u1[q + nx] + a.u1[q + nx + 1]);
        a.workV[p] = uV;
    }
    if (a.mU[p] == 1) a.ru[p] = drag<C>(a.u1[p], vU, a.DU[p], a.z0bU[p]);
    if (a.mV[p] == 1) a.rv[p] = drag<C>(uV, a.v1[p], a.DV[p], a.z0bV[p]);
}

// Momentum.coriolis, DEFAULT scheme (momentum.py:1127-1148): interp_xy of the
// transport to the other velocity grid, times f, negated for the V equation.
// (ioff, joff) are the interp_xy offsets: U -> V (1, 0); V -> U (0, 1).
__global__ void __launch_bounds__(S2_THREADS) coriolis_2d_kernel(int nx, int ny, int ioff, int joff,
                                                                  const double* src, const double* cor,
                                                                  double* out, int negate)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= nx || j >= ny) return;
    const long long p = (long long)j * nx + i;
    const int si = i - ioff, sj = j - joff;
    double v = out[p];
    if (si >= 0 && sj >= 0 && si <= nx - 2 && sj <= ny - 2) {
        const long long q = (long long)sj * nx + si;
        v = 0.25 * (src[q] + src[q + 1] + src[q + nx] + src[q + nx + 1]);
    }
    v = v * cor[p];
    out[p] = negate ? -v : v;
}

// Momentum.advance_depth_integrated's transport update, mixed form
// (momentum.F90:147-189): the tendency is summed in float, the transport is
// updated in double, and the implicit friction factor 1/(1 + x), x =
// dt r / D, is applied as U - U x/(1 + x) with the small correction in float
// (no FP64 division).
__global__ void __launch_bounds__(S2_THREADS) advance_2d_transport_mixed_kernel(
    int nx, int ny, int halox, int haloy, const int* mask, const double* alpha, const double* D,
    const double* dp, const double* taus, const double* cor, const double* adv, const double* diff,
    const double* damp, const double* SA, const double* SB, const double* SD, const double* SF,
    const double* r, double dt, double* U)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i < halox || i >= nx - halox || j < haloy || j >= ny - haloy) return;
    const long long p = (long long)j * nx + i;
    if (mask[p] != 1) return;
    const float rho0i = (float)(1.0 / GETM_RHO0);
    const double Up = U[p];
    const float sf = getm_d2f_approx(SF[p]);
    const float Slr = (Up > 0.0) ? fminf(sf, 0.f) : fmaxf(sf, 0.f);
    const float Dp = getm_d2f_approx(D[p]);
    const float dtf = (float)dt;
    const float tend = -(float)GETM_G * Dp * getm_d2f_approx(dp[p]) +
                       getm_d2f_approx(alpha[p]) *
                           (getm_d2f_approx(taus[p]) * rho0i + getm_d2f_approx(cor[p]) + getm_d2f_approx(adv[p]) +
                            getm_d2f_approx(diff[p]) + getm_d2f_approx(damp[p]) + getm_d2f_approx(SA[p]) +
                            getm_d2f_approx(SB[p]) + getm_d2f_approx(SD[p]) + Slr);
    const double num = Up + getm_f2d(dtf * tend);
    const float x = dtf * getm_d2f_approx(r[p]) / Dp;
    U[p] = num - getm_f2d(getm_d2f_approx(num) * (x / (1.f + x)));
}

// _U_cum += U; _V_cum += V (momentum.py:716-718), every point
__global__ void accumulate_2d_kernel(long long n, const double* U, const double* V, double* Uc, double* Vc)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    Uc[p] = Uc[p] + U[p];
    Vc[p] = Vc[p] + V[p];
}

// zo = z (every point), then the surface elevation update
// (simulation.py:1468-1486 -> wrapper.F90:496-523)
__global__ void __launch_bounds__(S2_THREADS) surface_elevation_fused_kernel(
    int nx, int ny, int halox, int haloy, const int* mask, const double* dyu, const double* dxv,
    const double* iarea, double* z, double* zo, const double* U, const double* V, const double* fwf, double dt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= nx || j >= ny) return;
    const long long p = (long long)j * nx + i;
    const double zp = z[p];
    zo[p] = zp;
    if (i < halox || i >= nx - halox || j < haloy || j >= ny - haloy) return;
    if (mask[p] != 1) return;
    z[p] = zp + dt * ((U[p - 1] * dyu[p - 1] - U[p] * dyu[p] + V[p - nx] * dxv[p - nx] - V[p] * dxv[p]) * iarea[p] + fwf[p]);
}

}  // namespace

static inline dim3 plane_grid(int nx, int ny) { return dim3(getm_div_up(nx, S2_THREADS), ny); }

extern "C" int getm_update_depth_2d(int nx, int ny, double Dmin, double Dcrit, const double* z, const double* zo,
                                    const double* HT, const double* HU, const double* HV, const double* HX,
                                    const int* mT, const int* mU, const int* mV, const int* mX, double* DT,
                                    double* DclipT, double* workT, double* workU, double* DU, double* alphaU,
                                    double* workV, double* DV, double* alphaV, double* workX, double* DX,
                                    double* DUU, double* DVV, double* DUV, double* DVU, cudaStream_t stream)
{
    if (nx < 2 || ny < 2) return GETM_ERR_ARG;
    const void* ptrs[] = {z, zo, HT, HU, HV, HX, mT, mU, mV, mX, DT, DclipT, workT, workU, DU, alphaU,
                          workV, DV, alphaV, workX, DX, DUU, DVV, DUV, DVU};
    for (const void* q : ptrs)
        if (!q) return GETM_ERR_ARG;
    DepthArgs a{nx, ny, Dmin, Dcrit, 1.0 / (Dcrit - 2 * Dmin), z, zo, HT, HU, HV, HX, mT, mU, mV, mX, DT, DclipT,
                workT, workU, DU, alphaU, workV, DV, alphaV, workX, DX, DUU, DVV, DUV, DVU};
    dim3 block(UD_BX, UD_BY);
    dim3 grid(getm_div_up(nx + 1, UD_BX), getm_div_up(ny + 1, UD_BY));
    update_depth_2d_kernel<<<grid, block, 0, stream>>>(a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_momentum_2d_velocities(int nx, int ny, int mixed, const double* U, const double* V,
                                           const double* DU, const double* DV, const double* DUU,
                                           const double* DUV, const double* DVU, const double* DVV, double* u1,
                                           double* v1, double* advU, double* advV, double* uua, double* uva,
                                           double* vua, double* vva, cudaStream_t stream)
{
    if (nx < 2 || ny < 2) return GETM_ERR_ARG;
    const void* ptrs[] = {U, V, DU, DV, DUU, DUV, DVU, DVV, u1, v1, advU, advV, uua, uva, vua, vva};
    for (const void* q : ptrs)
        if (!q) return GETM_ERR_ARG;
    VelArgs a{nx, ny, U, V, DU, DV, DUU, DUV, DVU, DVV, u1, v1, advU, advV, uua, uva, vua, vva};
    if (mixed) momentum_2d_velocities_kernel<float><<<plane_grid(nx, ny), S2_THREADS, 0, stream>>>(a);
    else momentum_2d_velocities_kernel<double><<<plane_grid(nx, ny), S2_THREADS, 0, stream>>>(a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_momentum_2d_friction(int nx, int ny, int mixed, const int* mU, const int* mV, const double* u1,
                                         const double* v1, const double* DU, const double* DV, const double* z0bU,
                                         const double* z0bV, double* workU, double* workV, double* ru, double* rv,
                                         cudaStream_t stream)
{
    if (nx < 2 || ny < 2) return GETM_ERR_ARG;
    const void* ptrs[] = {mU, mV, u1, v1, DU, DV, z0bU, z0bV, workU, workV, ru, rv};
    for (const void* q : ptrs)
        if (!q) return GETM_ERR_ARG;
    FricArgs a{nx, ny, mU, mV, u1, v1, DU, DV, z0bU, z0bV, workU, workV, ru, rv};
    if (mixed) momentum_2d_friction_kernel<float><<<plane_grid(nx, ny), S2_THREADS, 0, stream>>>(a);
    else momentum_2d_friction_kernel<double><<<plane_grid(nx, ny), S2_THREADS, 0, stream>>>(a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_coriolis_2d(int nx, int ny, int ioffset, int joffset, const double* src, const double* cor,
                                double* out, int negate, cudaStream_t stream)
{
    if (nx < 2 || ny < 2 || !src || !cor || !out || ioffset < 0 || ioffset > 1 || joffset < 0 || joffset > 1)
        return GETM_ERR_ARG;
    coriolis_2d_kernel<<<plane_grid(nx, ny), S2_THREADS, 0, stream>>>(nx, ny, ioffset, joffset, src, cor, out, negate);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_advance_2d_transport_mixed(int nx, int ny, int halox, int haloy, const int* mask,
                                               const double* alpha, const double* D, const double* dp,
                                               const double* taus, const double* cor, const double* adv,
                                               const double* diff, const double* damp, const double* SA,
                                               const double* SB, const double* SD, const double* SF,
                                               const double* r, double dt, double* U, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || !mask || !alpha || !D || !dp || !taus || !cor || !adv || !diff || !damp || !SA || !SB ||
        !SD || !SF || !r || !U)
        return GETM_ERR_ARG;
    advance_2d_transport_mixed_kernel<<<plane_grid(nx, ny), S2_THREADS, 0, stream>>>(
        nx, ny, halox, haloy, mask, alpha, D, dp, taus, cor, adv, diff, damp, SA, SB, SD, SF, r, dt, U);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_accumulate_2d(long long n, const double* U, const double* V, double* Ucum, double* Vcum,
                                  cudaStream_t stream)
{
    if (n < 0 || (n > 0 && (!U || !V || !Ucum || !Vcum))) return GETM_ERR_ARG;
    if (n == 0) return GETM_OK;
    accumulate_2d_kernel<<<getm_div_up(n, 256), 256, 0, stream>>>(n, U, V, Ucum, Vcum);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_surface_elevation_fused(int nx, int ny, int halox, int haloy, const int* mask,
                                            const double* dyu, const double* dxv, const double* iarea, double* z,
                                            double* zo, const double* U, const double* V, const double* fwf,
                                            double dt, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || halox < 1 || haloy < 1 || !mask || !dyu || !dxv || !iarea || !z || !zo || !U || !V || !fwf)
        return GETM_ERR_ARG;
    surface_elevation_fused_kernel<<<plane_grid(nx, ny), S2_THREADS, 0, stream>>>(nx, ny, halox, haloy, mask, dyu, dxv,
                                                                                   iarea, z, zo, U, V, fwf, dt);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}
