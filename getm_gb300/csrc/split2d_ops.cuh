// Point and tile functions of the split-explicit 2D substep, shared by the
// one-operation kernels (split2d.cu, momentum.cu, grid_ops.cu) and the
// persistent substep kernel (substep2d.cu), so that every operation has a
// single definition and both paths give the same results bit for bit.
//
// Layout: every field is [j][i] with the full halo-inclusive extents of its
// grid (nx_, ny_ for T, U, V and their velocity grids, nx_+1, ny_+1 for X).
#pragma once

#include <math.h>

#include <type_traits>

#include "getm_common.cuh"


// torch.clamp(x, min=lo): NaN propagates
__device__ __forceinline__ double clamp_min(double x, double lo) { return isnan(x) ? x : (x < lo ? lo : x); }

// The same values with the comparisons on the integer pipe (I: the mixed
// form) or on the FP64 pipe (the FP64 form, as written in the reference)
template <bool I>
__device__ __forceinline__ double dmax(double a, double b)
{
    if constexpr (I) return getm_fmax_i(a, b);
    else return fmax(a, b);
}

template <bool I>
__device__ __forceinline__ double dmin(double a, double b)
{
    if constexpr (I) return getm_fmin_i(a, b);
    else return fmin(a, b);
}

template <bool I>
__device__ __forceinline__ double dclamp_min(double x, double lo)
{
    if constexpr (I) return getm_isnan_i(x) ? x : (getm_dkey(x) < getm_dkey(lo) ? lo : x);
    else return clamp_min(x, lo);
}

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

constexpr int UD_BX = 32;  // tile width of update_depth_2d_tile

// alpha (wrapper.F90:428-436) with the constant divisor as a reciprocal
__device__ __forceinline__ double alpha_of(double d, double twoDmin, double ialpha)
{
    return fmax(0.0, fmin(1.0, (d - twoDmin) * ialpha));
}

// ... in float, for the mixed form: alpha is a weight between 0 and 1 that
// the mixed transport update reads as a float
__device__ __forceinline__ double alpha_of_f(double d, float twoDmin, float ialpha)
{
    return getm_f2d(fmaxf(0.f, fminf(1.f, (getm_d2f_approx(d) - twoDmin) * ialpha)));
}

// Simulation.update_depth, 2D part (simulation.py:1498-1586 without the
// halo exchanges and mirroring of a single closed domain).  A 32 x BY block
// covers X points (j, i) of its tile and the T, U, V points with the same
// indices; z_T_half of the tile plus a one-point halo is formed once into
// shared memory.  Copies between grids are scattered by the point that
// owns the source value (UU.D(j, i-1) = D_T_half(j, i), VV.D(j-1, i) =
// D_T_half(j, i), UV.D(j-1, i-1) = VU.D(j-1, i-1) = X.D(j, i)).
// MIXED: minima, maxima and clamps on the integer pipe (the same values) and
// alpha in float (alpha_of_f); the sums stay FP64.
template <int BY, bool MIXED = false>
__device__ __forceinline__ void update_depth_2d_tile(const DepthArgs& a, int bx, int by, int tx, int ty,
                                                     double (&szh)[BY + 2][UD_BX + 2])
{
    // szh: z_T_half at rows j0-1.., cols i0-1..
    const int i0 = bx * UD_BX, j0 = by * BY;
    const int i = i0 + tx, j = j0 + ty;
    const int nx = a.nx, ny = a.ny;
    // the point's own operands, loaded while the tile is staged
    const bool xin = i <= nx && j <= ny, tin = i < nx && j < ny;
    const long long px = (long long)j * (nx + 1) + i;
    const long long p = (long long)j * nx + i;
    int mX = 0, mT = 0, mU = 0, mV = 0;
    double workX0 = 0.0, DX0 = 0.0, HX = 0.0, DT0 = 0.0, HT = 0.0, zT = 0.0, workU0 = 0.0, HU = 0.0;
    double workV0 = 0.0, HV = 0.0;
    if (xin) {
        mX = a.mX[px]; workX0 = a.workX[px]; DX0 = a.DX[px]; HX = a.HX[px];
    }
    if (tin) {
        mT = a.mT[p]; DT0 = a.DT[p]; HT = a.HT[p]; zT = a.z[p];
        mU = a.mU[p]; workU0 = a.workU[p]; HU = a.HU[p];
        mV = a.mV[p]; workV0 = a.workV[p]; HV = a.HV[p];
    }
    for (int q = ty * UD_BX + tx; q < (BY + 2) * (UD_BX + 2); q += UD_BX * BY) {
        const int sj = q / (UD_BX + 2), si = q - sj * (UD_BX + 2);
        const int gj = j0 - 1 + sj, gi = i0 - 1 + si;
        double v = 0.0;
        if (gj >= 0 && gj < ny && gi >= 0 && gi < nx) {
            const long long g = (long long)gj * nx + gi;
            v = getm_half(a.zo[g] + a.z[g]);
        }
        szh[sj][si] = v;
    }
    __syncthreads();
    if (!xin) return;
    const int sj = ty + 1, si = tx + 1;  // (j, i) in the tile
    // X point (j, i): interp_xy T->X (offsets 1, 1) where it writes, else the
    // previous X._work value
    {
        double zx;
        if (j >= 1 && j <= ny - 1 && i >= 1 && i <= nx - 1) {
            zx = getm_quarter(szh[sj - 1][si - 1] + szh[sj - 1][si] + szh[sj][si - 1] + szh[sj][si]);
            a.workX[px] = zx;
        } else {
            zx = workX0;
        }
        double dx = DX0;
        if (mX != 0) {
            dx = dmax<MIXED>(HX + zx, a.Dmin);
            a.DX[px] = dx;
        }
        if (j >= 1 && i >= 1 && j - 1 < ny && i - 1 < nx) {  // UV.D = X.D[1:, 1:]; VU.D = UV.D
            const long long q = (long long)(j - 1) * nx + (i - 1);
            a.DUV[q] = dx;
            a.DVU[q] = dx;
        }
    }
    if (!tin) return;
    const double zh = szh[sj][si];
    // T: elevation2depth(z, H, -1000), Dclip = clamp(D, Dmin), D_T_half
    double DT = DT0;
    if (mT != 0) DT = dmax<MIXED>(HT + zT, -1000.0);
    a.DT[p] = DT;
    a.DclipT[p] = dclamp_min<MIXED>(DT, a.Dmin);
    const double dth = mT != 0 ? dmax<MIXED>(HT + zh, a.Dmin) : zh;
    a.workT[p] = dth;
    if (i >= 1) a.DUU[p - 1] = dth;   // UU.D[:, :-1] = D_T_half[:, 1:]
    if (j >= 1) a.DVV[p - nx] = dth;  // VV.D[:-1, :] = D_T_half[1:, :]
    const double twoDmin = 2 * a.Dmin;
    const float twoDmin_f = 2.f * getm_d2f_approx(a.Dmin), ialpha_f = getm_d2f_approx(a.ialpha);
    // U: z_U = interp_x(z_T_half, ioffset 0) for i < nx-1, else the old value
    double zu;
    if (i < nx - 1) {
        zu = getm_half(zh + szh[sj][si + 1]);
        a.workU[p] = zu;
    } else {
        zu = workU0;
    }
    if (mU != 0) {
        const double d = dmax<MIXED>(HU + zu, a.Dmin);
        a.DU[p] = d;
        a.alphaU[p] = MIXED ? alpha_of_f(d, twoDmin_f, ialpha_f) : alpha_of(d, twoDmin, a.ialpha);
    }
    // V: z_V = interp_y(z_T_half, joffset 0) for j < ny-1
    double zv;
    if (j < ny - 1) {
        zv = getm_half(zh + szh[sj + 1][si]);
        a.workV[p] = zv;
    } else {
        zv = workV0;
    }
    if (mV != 0) {
        const double d = dmax<MIXED>(HV + zv, a.Dmin);
        a.DV[p] = d;
        a.alphaV[p] = MIXED ? alpha_of_f(d, twoDmin_f, ialpha_f) : alpha_of(d, twoDmin, a.ialpha);
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

// Mixed form: u1 = U/D to ~2^-46 (getm_div_refined; u1 is advected and its
// product with the new depth is differenced against U, so it stays FP64) and
// the advection velocities entirely in float.
template <typename C>
__device__ __forceinline__ void momentum_2d_velocities_point(const VelArgs& a, int i, int j)
{
    const long long p = (long long)j * a.nx + i;
    if constexpr (std::is_same<C, double>::value) {
        const double u1 = a.U[p] / a.DU[p];
        const double v1 = a.V[p] / a.DV[p];
        a.u1[p] = u1; a.advU[p] = u1;
        a.v1[p] = v1; a.advV[p] = v1;
        // interp_x (ioffset 0) writes i < nx-1; elsewhere the old value is divided
        const double uu = i < a.nx - 1 ? getm_half(a.U[p] + a.U[p + 1]) : a.uua[p];
        const double uv = i < a.nx - 1 ? getm_half(a.V[p] + a.V[p + 1]) : a.uva[p];
        const double vu = j < a.ny - 1 ? getm_half(a.U[p] + a.U[p + a.nx]) : a.vua[p];
        const double vv = j < a.ny - 1 ? getm_half(a.V[p] + a.V[p + a.nx]) : a.vva[p];
        a.uua[p] = vel_div<C>(uu, a.DUU[p]);
        a.uva[p] = vel_div<C>(uv, a.DUV[p]);
        a.vua[p] = vel_div<C>(vu, a.DVU[p]);
        a.vva[p] = vel_div<C>(vv, a.DVV[p]);
    } else {
        const double Up = a.U[p], Vp = a.V[p];
        const double u1 = getm_div_refined(Up, a.DU[p]);
        const double v1 = getm_div_refined(Vp, a.DV[p]);
        a.u1[p] = u1; a.advU[p] = u1;
        a.v1[p] = v1; a.advV[p] = v1;
        const float Uf = getm_d2f_approx(Up), Vf = getm_d2f_approx(Vp);
        const float uu = i < a.nx - 1 ? 0.5f * (Uf + getm_d2f_approx(a.U[p + 1])) : getm_d2f_approx(a.uua[p]);
        const float uv = i < a.nx - 1 ? 0.5f * (Vf + getm_d2f_approx(a.V[p + 1])) : getm_d2f_approx(a.uva[p]);
        const float vu = j < a.ny - 1 ? 0.5f * (Uf + getm_d2f_approx(a.U[p + a.nx])) : getm_d2f_approx(a.vua[p]);
        const float vv = j < a.ny - 1 ? 0.5f * (Vf + getm_d2f_approx(a.V[p + a.nx])) : getm_d2f_approx(a.vva[p]);
        a.uua[p] = getm_f2d(uu / getm_d2f_approx(a.DUU[p]));
        a.uva[p] = getm_f2d(uv / getm_d2f_approx(a.DUV[p]));
        a.vua[p] = getm_f2d(vu / getm_d2f_approx(a.DVU[p]));
        a.vva[p] = getm_f2d(vv / getm_d2f_approx(a.DVV[p]));
    }
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
__device__ __forceinline__ C to_c(double x)
{
    if constexpr (std::is_same<C, double>::value) return x;
    else return getm_d2f_approx(x);
}

template <typename C>
__device__ __forceinline__ double from_c(C x)
{
    if constexpr (std::is_same<C, double>::value) return x;
    else return getm_f2d(x);
}

template <typename C>
__device__ __forceinline__ double drag(C uu, C vv, double D, double z0)
{
    const C DD = to_c<C>(D);
    const C sqrtcd = C(GETM_KAPPA) / log(C(1) + C(0.5) * DD / to_c<C>(z0));
    return from_c<C>(sqrtcd * sqrtcd * sqrt(getm_speed2(uu, vv)));
}

template <typename C>
__device__ __forceinline__ void momentum_2d_friction_point(const FricArgs& a, int i, int j)
{
    const long long p = (long long)j * a.nx + i;
    const int nx = a.nx;
    // the point's own operands, loaded before any mask is tested
    const int mU = a.mU[p], mV = a.mV[p];
    const double u1p = a.u1[p], v1p = a.v1[p], DUp = a.DU[p], DVp = a.DV[p], z0bUp = a.z0bU[p], z0bVp = a.z0bV[p];
    // v_U = interp_xy(v1, ioffset 0, joffset 1): written at j >= 1, i <= nx-2
    // (in arithmetic C: the drag coefficient is evaluated in C)
    C vU;
    if (j >= 1 && i <= nx - 2) {
        const long long q = p - nx;
        vU = C(0.25) * (to_c<C>(a.v1[q]) + to_c<C>(a.v1[q + 1]) + to_c<C>(a.v1[q + nx]) + to_c<C>(a.v1[q + nx + 1]));
        a.workU[p] = from_c<C>(vU);
    } else {
        vU = to_c<C>(a.workU[p]);
    }
    // u_V = interp_xy(u1, ioffset 1, joffset 0): written at i >= 1, j <= ny-2
    C uV;
    if (i >= 1 && j <= a.ny - 2) {
        const long long q = p - 1;
        uV = C(0.25) * (to_c<C>(a.u1[q]) + to_c<C>(a.u1[q + 1]) + to_c<C>(a.u1[q + nx]) + to_c<C>(a.u1[q + nx + 1]));
        a.workV[p] = from_c<C>(uV);
    } else {
        uV = to_c<C>(a.workV[p]);
    }
    if (mU == 1) a.ru[p] = drag<C>(to_c<C>(u1p), vU, DUp, z0bUp);
    if (mV == 1) a.rv[p] = drag<C>(uV, to_c<C>(v1p), DVp, z0bVp);
}

// Momentum.coriolis, DEFAULT scheme (momentum.py:1127-1148): interp_xy of the
// transport to the other velocity grid, times f, negated for the V equation.
// (ioff, joff) are the interp_xy offsets: U -> V (1, 0); V -> U (0, 1).
// C: arithmetic (float in the mixed form, whose transport update reads the
// term as a float tendency).
// true where the interpolation writes point (i, j) of the target grid
__device__ __forceinline__ bool coriolis_2d_inside(int nx, int ny, int ioff, int joff, int i, int j)
{
    const int si = i - ioff, sj = j - joff;
    return si >= 0 && sj >= 0 && si <= nx - 2 && sj <= ny - 2;
}

// The term at (i, j) inside the interpolation range; src(i, j) returns the
// transport at a source point.
template <typename C, typename Src>
__device__ __forceinline__ double coriolis_2d_value(int ioff, int joff, int i, int j, const Src& src, double cor,
                                                    int negate)
{
    const int si = i - ioff, sj = j - joff;
    C v = C(0.25) * (to_c<C>(src(si, sj)) + to_c<C>(src(si + 1, sj)) + to_c<C>(src(si, sj + 1)) +
                     to_c<C>(src(si + 1, sj + 1)));
    v = v * to_c<C>(cor);
    return from_c<C>(negate ? -v : v);
}

// ... and outside it (the previous value times f)
template <typename C>
__device__ __forceinline__ double coriolis_2d_outside(double old, double cor, int negate)
{
    C v = to_c<C>(old);
    v = v * to_c<C>(cor);
    return from_c<C>(negate ? -v : v);
}

template <typename C>
__device__ __forceinline__ void coriolis_2d_point(int nx, int ny, int ioff, int joff, const double* src,
                                                  const double* cor, double* out, int negate, int i, int j)
{
    const long long p = (long long)j * nx + i;
    if (coriolis_2d_inside(nx, ny, ioff, joff, i, j)) {
        auto at = [&](int si, int sj) { return src[(long long)sj * nx + si]; };
        out[p] = coriolis_2d_value<C>(ioff, joff, i, j, at, cor[p], negate);
    } else {
        out[p] = coriolis_2d_outside<C>(out[p], cor[p], negate);
    }
}

// Momentum.advance_depth_integrated's transport update (momentum.F90:147-189)
// at interior point p; a: the fields of one direction (U or V).
struct Transport2DArgs {
    const int* mask;
    const double *alpha, *D, *dp, *taus, *cor, *adv, *diff, *damp, *SA, *SB, *SD, *SF, *r;
    double* U;
};

// The transport after the update at interior point p: the new value where
// the mask is 1, else the old one (upd false).  cor: the Coriolis term at p.
// Every operand is loaded before the mask is tested (one round of
// independent loads per point).
struct TransportNew {
    double v;
    bool upd;
};

__device__ __forceinline__ TransportNew transport_2d_value(const Transport2DArgs& a, double dt, long long p,
                                                           double cor)
{
    const int m = a.mask[p];
    const double Up = a.U[p], SF = a.SF[p], Dp = a.D[p], dp = a.dp[p], alpha = a.alpha[p], taus = a.taus[p];
    const double adv = a.adv[p], diff = a.diff[p], damp = a.damp[p];
    const double SA = a.SA[p], SB = a.SB[p], SD = a.SD[p], r = a.r[p];
    if (m != 1) return TransportNew{Up, false};
    const double rho0i = 1.0 / GETM_RHO0;
    double Slr = (Up > 0.0) ? fmin(SF, 0.0) : fmax(SF, 0.0);
    return TransportNew{(Up + dt * (-GETM_G * Dp * dp + alpha * (taus * rho0i + cor + adv + diff + damp + SA + SB + SD + Slr)))
                            / (1.0 + dt * r / Dp),
                        true};
}

__device__ __forceinline__ void transport_2d_point(const Transport2DArgs& a, double dt, long long p)
{
    const TransportNew n = transport_2d_value(a, dt, p, a.cor[p]);
    if (n.upd) a.U[p] = n.v;
}

// Momentum.advance_depth_integrated's transport update, mixed form
// (momentum.F90:147-189): the tendency is summed in float, the transport is
// updated in double, and the implicit friction factor 1/(1 + x), x =
// dt r / D, is applied as U - U x/(1 + x) with the small correction in float
// (no FP64 division).
__device__ __forceinline__ TransportNew transport_2d_mixed_value(const Transport2DArgs& a, double dt, long long p,
                                                                 double corp)
{
    const int* mask = a.mask;
    const double *alpha = a.alpha, *D = a.D, *dp = a.dp, *taus = a.taus, *adv = a.adv;
    const double *diff = a.diff, *damp = a.damp, *SA = a.SA, *SB = a.SB, *SD = a.SD, *SF = a.SF, *r = a.r;
    const int m = mask[p];
    const double Up = a.U[p], SFp = SF[p], Dd = D[p], dpp = dp[p], alp = alpha[p], tau = taus[p];
    const double advp = adv[p], diffp = diff[p], dampp = damp[p], SAp = SA[p], SBp = SB[p], SDp = SD[p], rp = r[p];
    if (m != 1) return TransportNew{Up, false};
    const float rho0i = (float)(1.0 / GETM_RHO0);
    const float sf = getm_d2f_approx(SFp);
    const float Slr = getm_positive_i(Up) ? fminf(sf, 0.f) : fmaxf(sf, 0.f);
    const float Dp = getm_d2f_approx(Dd);
    const float dtf = (float)dt;
    const float tend = -(float)GETM_G * Dp * getm_d2f_approx(dpp) +
                       getm_d2f_approx(alp) *
                           (getm_d2f_approx(tau) * rho0i + getm_d2f_approx(corp) + getm_d2f_approx(advp) +
                            getm_d2f_approx(diffp) + getm_d2f_approx(dampp) + getm_d2f_approx(SAp) +
                            getm_d2f_approx(SBp) + getm_d2f_approx(SDp) + Slr);
    const double num = Up + getm_f2d(dtf * tend);
    const float x = dtf * getm_d2f_approx(rp) / Dp;
    return TransportNew{num - getm_f2d(getm_d2f_approx(num) * (x / (1.f + x))), true};
}

__device__ __forceinline__ void transport_2d_mixed_point(const Transport2DArgs& a, double dt, long long p)
{
    const TransportNew n = transport_2d_mixed_value(a, dt, p, a.cor[p]);
    if (n.upd) a.U[p] = n.v;
}

// _U_cum += U; _V_cum += V (momentum.py:716-718), every point
__device__ __forceinline__ void accumulate_2d_point(const double* U, const double* V, double* Uc, double* Vc,
                                                    long long p)
{
    Uc[p] = Uc[p] + U[p];
    Vc[p] = Vc[p] + V[p];
}

// zo = z (every point), then the surface elevation update
// (simulation.py:1468-1486 -> wrapper.F90:496-523)
// the elevation update at an interior water point (wrapper.F90:496-523)
__device__ __forceinline__ double elevation_new(double zp, double dt, double Uw, double dyw, double Ue, double dye,
                                                double Vs, double dxs, double Vn, double dxn, double ia, double fw)
{
    return zp + dt * ((Uw * dyw - Ue * dye + Vs * dxs - Vn * dxn) * ia + fw);
}

__device__ __forceinline__ void surface_elevation_fused_point(int nx, int ny, int halox, int haloy, const int* mask,
                                                              const double* dyu, const double* dxv,
                                                              const double* iarea, double* z, double* zo,
                                                              const double* U, const double* V, const double* fwf,
                                                              double dt, int i, int j)
{
    const long long p = (long long)j * nx + i;
    const double zp = z[p];
    zo[p] = zp;
    if (i < halox || i >= nx - halox || j < haloy || j >= ny - haloy) return;
    // every operand is loaded before the mask is tested
    const int m = mask[p];
    const double Uw = U[p - 1], dyw = dyu[p - 1], Ue = U[p], dye = dyu[p], Vs = V[p - nx], dxs = dxv[p - nx];
    const double Vn = V[p], dxn = dxv[p], ia = iarea[p], fw = fwf[p];
    if (m != 1) return;
    z[p] = elevation_new(zp, dt, Uw, dyw, Ue, dye, Vs, dxs, Vn, dxn, ia, fw);
}


// reconstruct_transport_change (momentum.F90:323-340) at point p of a row
// inside jmin..jmax (T: type of un and Uo)
template <typename T>
__device__ __forceinline__ void reconstruct_point(T* un, const double* hn, const T* Uo, double idt, long long p)
{
    if constexpr (std::is_same<T, double>::value) un[p] = (un[p] * hn[p] - Uo[p]) * idt;
    else un[p] = (un[p] * getm_d2f_approx(hn[p]) - Uo[p]) * (T)idt;
}

// surface_pressure_gradient (wrapper.F90:525-565) at interior point (i, j)
struct SpgArgs {
    int nx;
    const int *umask, *vmask;
    const double *idxu, *idyv, *z, *sp, *H, *D;
    double Dmin;
    double *dpdx, *dpdy;
};

// MIXED: the elevation bounds on the integer pipe, the two differences in
// FP64 and the rest in float (the mixed transport update reads the gradient
// as a float).
template <bool MIXED = false>
__device__ __forceinline__ void spg_point(const SpgArgs& a, long long p)
{
    const int nx = a.nx;
    const double gammai = 1.0 / (GETM_G * GETM_RHO0);
    // every operand is loaded before the masks are tested
    const int mu = a.umask[p], mv = a.vmask[p];
    const double z0 = a.z[p], z1 = a.z[p + 1], zn = a.z[p + nx];
    const double H0 = a.H[p], H1 = a.H[p + 1], Hn = a.H[p + nx];
    const double D0 = a.D[p], D1 = a.D[p + 1], Dn = a.D[p + nx];
    const double sp0 = a.sp[p], sp1 = a.sp[p + 1], spn = a.sp[p + nx];
    const double idx = a.idxu[p], idy = a.idyv[p];
    if constexpr (MIXED) {
        const float gi = (float)(1.0 / (GETM_G * GETM_RHO0));
        if (mu == 1) {
            const double zp = getm_fmax_i(z1, -H0 + getm_fmin_i(a.Dmin, D1));
            const double zm = getm_fmax_i(z0, -H1 + getm_fmin_i(a.Dmin, D0));
            const float g = getm_d2f_approx(zp - zm) + getm_d2f_approx(sp1 - sp0) * gi;
            a.dpdx[p] = getm_f2d(g * getm_d2f_approx(idx));
        }
        if (mv == 1) {
            const double zp = getm_fmax_i(zn, -H0 + getm_fmin_i(a.Dmin, Dn));
            const double zm = getm_fmax_i(z0, -Hn + getm_fmin_i(a.Dmin, D0));
            const float g = getm_d2f_approx(zp - zm) + getm_d2f_approx(spn - sp0) * gi;
            a.dpdy[p] = getm_f2d(g * getm_d2f_approx(idy));
        }
        return;
    }
    if (mu == 1) {
        double zp = fmax(z1, -H0 + fmin(a.Dmin, D1));
        double zm = fmax(z0, -H1 + fmin(a.Dmin, D0));
        a.dpdx[p] = (zp - zm + (sp1 - sp0) * gammai) * idx;
    }
    if (mv == 1) {
        double zp = fmax(zn, -H0 + fmin(a.Dmin, Dn));
        double zm = fmax(z0, -Hn + fmin(a.Dmin, D0));
        a.dpdy[p] = (zp - zm + (spn - sp0) * gammai) * idy;
    }
}

// interp_x / interp_y (interpolation.F90:9-40) of one point: t = mean of s
// at p and its neighbour at +step, stored at p + off (off = 0 or step)
template <typename T>
__device__ __forceinline__ void interp_pair_point(const T* s, T* t, long long p, long long step, long long off)
{
    t[p + off] = T(0.5) * (s[p] + s[p + step]);
}
