// Internal pressure gradients of python/src/internal_pressure.F90 for sm_103a:
// Blumberg & Mellor (:9-60) and Shchepetkin & McWilliams (:63-217).
//
// Blumberg-Mellor: one thread per water column integrates downward from the
// surface for the U and the V point of that column.
// Shchepetkin-McWilliams, two kernels:
//   1. thread per T column: vertical harmonic-mean slopes dR, dZ (kept in a
//      register window, never stored) and the column pressure integral P,
//      written to a caller-provided 3D work array;
//   2. thread per (i, j, k) U/V point: horizontal harmonic-mean slopes from
//      the three raw differences around the point, the density-Jacobian
//      correction FC and the gradient.  The reference's per-level dZx/dRx
//      work arrays are recomputed in registers (same operations, same values);
//      the mixed form forms each raw difference once per 32 x 8 tile in
//      shared memory.
#include "getm_common.cuh"

// ---------------------------------------------------------------------------
// Blumberg & Mellor
// ---------------------------------------------------------------------------
// T: type of buoyancy and of the gradients; the integration runs in FP64.
template <typename T>
__global__ void blumberg_mellor_kernel(int nx, int ny, int nz, int ilo, int ihi, int jlo, int jhi,
                                       const int* umask, const int* vmask, const double* idxu,
                                       const double* idyv, const double* hu, const double* hv,
                                       const double* zf, const T* buoy, T* idpdx, T* idpdy)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y + jlo;
    if (i < ilo || i > ihi || j > jhi) return;
    const long long P = (long long)nx * ny;
    const long long p = (long long)j * nx + i;
    // levels: buoy/hu Fortran k -> plane k-1; zf Fortran k -> plane k
    for (int dir = 0; dir < 2; dir++) {
        const int* m = dir ? vmask : umask;
        if (m[p] <= 0) continue;
        const long long s = dir ? nx : 1;
        const double id = dir ? idyv[p] : idxu[p];
        const double* hh = dir ? hv : hu;
        T* out = dir ? idpdy : idpdx;
        long long q = p + (long long)(nz - 1) * P;
        double grdl = ((double)buoy[q + s] - (double)buoy[q]) * id;
        double buoyl = 0.5 * ((double)buoy[q + s] + (double)buoy[q]);
        double hk1 = hh[q];
        double prgr = grdl * 0.5 * hk1;
        out[q] = (T)(hk1 * prgr);
        for (int k = nz - 1; k >= 1; k--) {
            q = p + (long long)(k - 1) * P;
            double grdu = grdl;
            grdl = ((double)buoy[q + s] - (double)buoy[q]) * id;
            double buoyu = buoyl;
            buoyl = 0.5 * ((double)buoy[q + s] + (double)buoy[q]);
            long long qf = p + (long long)k * P;
            double dxz = (zf[qf + s] - zf[qf]) * id;
            double hk = hh[q];
            prgr = prgr + 0.5 * (grdu + grdl) * 0.5 * (hk + hk1) - dxz * (buoyu - buoyl);
            out[q] = (T)(hk * prgr);
            hk1 = hk;
        }
    }
}

template <typename T>
static int bm_impl(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax, const int* umask,
                   const int* vmask, const double* idxu, const double* idyv, const double* hu, const double* hv,
                   const double* zf, const T* buoy, T* idpdx, T* idpdy, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || imin < 1 || jmin < 1 || imax >= nx || jmax >= ny || jmax < jmin) return GETM_ERR_ARG;
    if (!umask || !vmask || !idxu || !idyv || !hu || !hv || !zf || !buoy || !idpdx || !idpdy) return GETM_ERR_ARG;
    dim3 grid(getm_div_up(nx, 128), jmax - jmin + 1);
    blumberg_mellor_kernel<T><<<grid, 128, 0, stream>>>(nx, ny, nz, imin - 1, imax - 1, jmin - 1, jmax - 1, umask, vmask, idxu, idyv, hu, hv, zf, buoy, idpdx, idpdy);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_blumberg_mellor(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                                    const int* umask, const int* vmask, const double* idxu,
                                    const double* idyv, const double* hu, const double* hv,
                                    const double* zf, const double* buoy, double* idpdx, double* idpdy,
                                    cudaStream_t stream)
{
    return bm_impl<double>(nx, ny, nz, imin, imax, jmin, jmax, umask, vmask, idxu, idyv, hu, hv, zf, buoy, idpdx, idpdy, stream);
}

extern "C" int getm_blumberg_mellor_f32(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                                        const int* umask, const int* vmask, const double* idxu,
                                        const double* idyv, const double* hu, const double* hv,
                                        const double* zf, const float* buoy, float* idpdx, float* idpdy,
                                        cudaStream_t stream)
{
    return bm_impl<float>(nx, ny, nz, imin, imax, jmin, jmax, umask, vmask, idxu, idyv, hu, hv, zf, buoy, idpdx, idpdy, stream);
}

// ---------------------------------------------------------------------------
// Shchepetkin & McWilliams
// ---------------------------------------------------------------------------
#define SMCW_EPS 1.e-10

// Harmonic mean with the cut-off of internal_pressure.F90:93-98.
template <typename T>
__device__ __forceinline__ T smcw_harm_cut(T a, T b)
{
    T cff = T(2) * a * b;
    return (cff > T(SMCW_EPS)) ? cff / (a + b) : T(0);
}

// Phase 1 (internal_pressure.F90:80-118): column pressure integral P.
// Columns with mask > 0 over C i in [ilo, ihi+1], j in [jlo, jhi+1].
template <typename T>
__global__ void smcw_column_kernel(int nx, int ny, int nz, int ilo, int ihi, int jlo, int jhi,
                                   const int* mask, const double* h, const double* zc,
                                   const T* buoy, double* Pw)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y + jlo;
    if (i < ilo || i > ihi + 1 || j > jhi + 1) return;
    const long long P = (long long)nx * ny;
    const long long p = (long long)j * nx + i;
    if (mask[p] <= 0) return;
    const double x = 1.0 / 12.0;
#define B(k) ((double)buoy[p + (long long)((k) - 1) * P])
#define Z(k) zc[p + (long long)((k) - 1) * P]
    // Fortran levels 1..nz.  Raw differences d(k) = v(k+1) - v(k), k = 1..nz-1,
    // d(nz) = d(nz-1), d(0) = d(1); harmonic HR(k) from d(k), d(k-1).
    double cff = 0.0;
    if (nz > 1) cff = 0.5 * (B(nz) - B(nz - 1)) * 0.5 * h[p + (long long)(nz - 1) * P] / (Z(nz) - Z(nz - 1));
    double Pk = (B(nz) + cff) * 0.5 * h[p + (long long)(nz - 1) * P];
    Pw[p + (long long)(nz - 1) * P] = Pk;
    if (nz == 1) return;
    // window at level k+1 = nz: HR(nz) uses d(nz) = d(nz-1) and d(nz-1)
    double bk1 = B(nz), zk1 = Z(nz);          // v(k+1)
    double bk = B(nz - 1), zk = Z(nz - 1);    // v(k)
    double dRk = bk1 - bk, dZk = zk1 - zk;    // d(k) with k = nz-1
    double HR1 = smcw_harm_cut<double>(dRk, dRk);     // HR(nz): d(nz) = d(nz-1)
    double HZ1 = 2.0 * dZk * dZk / (dZk + dZk);
    for (int k = nz - 1; k >= 1; k--) {
        // d(k-1): for k == 1 it is d(0) = d(1)
        double dRm, dZm, bkm1 = 0.0, zkm1 = 0.0;
        if (k > 1) {
            bkm1 = B(k - 1); zkm1 = Z(k - 1);
            dRm = bk - bkm1; dZm = zk - zkm1;
        } else {
            dRm = dRk; dZm = dZk;
        }
        double HR0 = smcw_harm_cut<double>(dRk, dRm);   // HR(k)
        double HZ0 = 2.0 * dZk * dZm / (dZk + dZm);
        Pk = Pk + 0.5 * ((bk1 + bk) * (zk1 - zk) - 0.2 * ((HR1 - HR0) * (zk1 - zk - x * (HZ1 + HZ0))
                  - (HZ1 - HZ0) * (bk1 - bk - x * (HR1 + HR0))));
        Pw[p + (long long)(k - 1) * P] = Pk;
        // shift: level k becomes k+1
        HR1 = HR0; HZ1 = HZ0;
        bk1 = bk; zk1 = zk; bk = bkm1; zk = zkm1;
        dRk = dRm; dZk = dZm;
    }
#undef B
#undef Z
}

// Phase 2 (internal_pressure.F90:120-216), both directions (s = 1: x,
// s = nx: y).  T: type of buoyancy, of the gradients and of the slope
// arithmetic; height and pressure differences are formed in FP64 first.
template <typename T>
__global__ void smcw_gradient_kernel(int nx, int ny, int nz, int ilo, int ihi, int jlo, int jhi,
                                     const int* umask, const int* vmask, const double* idxu,
                                     const double* idyv, const double* h, const double* z,
                                     const double* zc, const T* buoy, const double* Pw,
                                     T* idpdx, T* idpdy)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y + jlo;
    int k = blockIdx.z;  // C level (Fortran k+1)
    if (i < ilo || i > ihi || j > jhi) return;
    const long long P = (long long)nx * ny;
    const long long p = (long long)j * nx + i;
    const long long q = p + (long long)k * P;
    const long long qtop = p + (long long)(nz - 1) * P;
    const T x = T(1.0) / T(12.0);
    for (int dir = 0; dir < 2; dir++) {
        const int* m = dir ? vmask : umask;
        if (m[p] != 1) continue;
        const long long s = dir ? nx : 1;
        // raw differences at p, p+s, p+2s (Fortran i, i+1, i+2), each gated
        // by the mask of the velocity point just before it
        T rZ0 = T(0), rR0 = T(0), rZ1 = T(0), rR1 = T(0), rZ2 = T(0), rR2 = T(0);
        if (m[p - s] > 0) { rZ0 = (T)(zc[q] - zc[q - s]); rR0 = buoy[q] - buoy[q - s]; }
        if (m[p] > 0) { rZ1 = (T)(zc[q + s] - zc[q]); rR1 = buoy[q + s] - buoy[q]; }
        if (m[p + s] > 0) { rZ2 = (T)(zc[q + 2 * s] - zc[q + s]); rR2 = buoy[q + 2 * s] - buoy[q + s]; }
        T dZx0 = smcw_harm_cut<T>(rZ0, rZ1), dZx1 = smcw_harm_cut<T>(rZ1, rZ2);
        T dRx0 = smcw_harm_cut<T>(rR0, rR1), dRx1 = smcw_harm_cut<T>(rR1, rR2);
        T dzc = (T)(zc[q + s] - zc[q]);
        T FC = T(0.5) * ((buoy[q + s] + buoy[q]) * dzc
               - T(0.2) * ((dRx1 - dRx0) * (dzc - x * (dZx1 + dZx0))
               - (dZx1 - dZx0) * (buoy[q + s] - buoy[q] - x * (dRx1 + dRx0))));
        double id = dir ? idyv[p] : idxu[p];
        T* out = dir ? idpdy : idpdx;
        out[q] = (T)(0.5 * (h[q] + h[q + s]) * id)
                 * ((T)(Pw[q + s] - Pw[q]) + FC - (T)(z[p + s] - z[p]) * T(0.5) * (buoy[qtop + s] + buoy[qtop]));
    }
}

// ---------------------------------------------------------------------------
// Mixed-form SMcW: double buoyancy, heights, pressure and gradients; the main
// terms (column sums of b dz, pressure differences, the hydrostatic
// correction) in FP64, the harmonic-mean slope corrections of
// internal_pressure.F90:93-99, :143-166 in float from FP64 differences.  The
// slopes are the divisions of the scheme, so this removes nearly all of its
// FP64 work while keeping the large, nearly cancelling terms in FP64.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float smcw_harm_f(float a, float b)
{
    const float cff = 2.f * a * b;
    return (cff > (float)SMCW_EPS) ? cff / (a + b) : 0.f;
}

// Pw: nz + 2 planes; the last two receive the hydrostatic surface term of
// the x and y gradients of the column, (z_e - z) (b_e + b)/2 at the top
// layer, formed once per column instead of once per layer.
__global__ void smcw_column_mixed_kernel(int nx, int ny, int nz, int ilo, int ihi, int jlo, int jhi,
                                         const int* __restrict__ mask, const double* __restrict__ h, const double* __restrict__ zc,
                                         const double* __restrict__ buoy, const double* __restrict__ z,
                                         double* __restrict__ Pw)
{
    int i, j;
    if (!getm_flat_column(nx, jlo, jhi - jlo + 2, i, j) || i < ilo || i > ihi + 1) return;
    const long long P = (long long)nx * ny;
    const long long p = (long long)j * nx + i;
    if (mask[p] <= 0) return;
    const float x = 1.f / 12.f;
    if (i <= ihi && j <= jhi) {
        const long long ptop = p + (long long)(nz - 1) * P;
        Pw[p + (long long)nz * P] = (z[p + 1] - z[p]) * 0.5 * (buoy[ptop + 1] + buoy[ptop]);
        Pw[p + (long long)(nz + 1) * P] = (z[p + nx] - z[p]) * 0.5 * (buoy[ptop + nx] + buoy[ptop]);
    }
#define B(k) buoy[p + (long long)((k) - 1) * P]
#define Z(k) zc[p + (long long)((k) - 1) * P]
    double cff = 0.0;
    if (nz > 1) cff = 0.5 * (B(nz) - B(nz - 1)) * 0.5 * h[p + (long long)(nz - 1) * P] / (Z(nz) - Z(nz - 1));
    double Pk = (B(nz) + cff) * 0.5 * h[p + (long long)(nz - 1) * P];
    Pw[p + (long long)(nz - 1) * P] = Pk;
    if (nz == 1) return;
    double bk1 = B(nz), zk1 = Z(nz);
    double bk = B(nz - 1), zk = Z(nz - 1);
    float dRk = getm_d2f_approx(bk1 - bk), dZk = getm_d2f_approx(zk1 - zk);
    float HR1 = smcw_harm_f(dRk, dRk);
    float HZ1 = 2.f * dZk * dZk / (dZk + dZk);
    for (int k = nz - 1; k >= 1; k--) {
        float dRm, dZm;
        double bkm1 = 0.0, zkm1 = 0.0;
        if (k > 1) {
            bkm1 = B(k - 1); zkm1 = Z(k - 1);
            dRm = getm_d2f_approx(bk - bkm1); dZm = getm_d2f_approx(zk - zkm1);
        } else {
            dRm = dRk; dZm = dZk;
        }
        const float HR0 = smcw_harm_f(dRk, dRm);
        const float HZ0 = 2.f * dZk * dZm / (dZk + dZm);
        const float corr = 0.2f * ((HR1 - HR0) * (dZk - x * (HZ1 + HZ0)) - (HZ1 - HZ0) * (dRk - x * (HR1 + HR0)));
        Pk = Pk + 0.5 * ((bk1 + bk) * (zk1 - zk) - getm_f2d(corr));
        Pw[p + (long long)(k - 1) * P] = Pk;
        HR1 = HR0; HZ1 = HZ0;
        bk1 = bk; zk1 = zk; bk = bkm1; zk = zkm1;
        dRk = dRm; dZk = dZm;
    }
#undef B
#undef Z
}

// Gradient, both directions, on 32 x SG_BY tiles of one level.  The raw
// differences between neighbouring points (zc and buoyancy, x and y, each
// gated by the mask of the velocity point between them) are formed once per
// face into shared memory instead of three times (once for each of the three
// points that use them); a point keeps the FP64 differences of its own faces
// for the density-Jacobian term.  The values are those of the per-point
// form, operation for operation.
constexpr int SG_BX = 32, SG_BY = 8;

struct SgFace {
    float rz, rr;   // gated float differences (zero where the mask is not positive)
    double dz, db;  // FP64 differences, valid where the mask is positive
};

__device__ __forceinline__ SgFace smcw_face(const int* __restrict__ m, long long p, long long q, long long s,
                                            const double* __restrict__ zc, const double* __restrict__ buoy)
{
    SgFace f{0.f, 0.f, 0.0, 0.0};
    if (m[p] > 0) {
        f.dz = zc[q + s] - zc[q];
        f.db = buoy[q + s] - buoy[q];
        f.rz = getm_d2f_approx(f.dz);
        f.rr = getm_d2f_approx(f.db);
    }
    return f;
}

__global__ void smcw_gradient_mixed_kernel(
    int nx, int ny, int nz, int ilo, int ihi, int jlo, int jhi, const int* __restrict__ umask,
    const int* __restrict__ vmask, const double* __restrict__ idxu, const double* __restrict__ idyv,
    const double* __restrict__ h, const double* __restrict__ zc, const double* __restrict__ buoy,
    const double* __restrict__ Pw, double* __restrict__ idpdx, double* __restrict__ idpdy)
{
    // x faces of columns i0-1 .. i0+SG_BX, y faces of rows j0-1 .. j0+SG_BY
    __shared__ float sZx[SG_BY][SG_BX + 2], sRx[SG_BY][SG_BX + 2];
    __shared__ float sZy[SG_BY + 2][SG_BX], sRy[SG_BY + 2][SG_BX];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = blockIdx.x * SG_BX, j0 = jlo + blockIdx.y * SG_BY;
    const int i = i0 + tx, j = j0 + ty;
    const int k = blockIdx.z;
    const long long P = (long long)nx * ny;
    const long long kP = (long long)k * P;
    const long long p = (long long)j * nx + i;
    // faces needed: x at columns ilo-1 .. ihi+1 of rows jlo .. jhi, y at
    // rows jlo-1 .. jhi+1 of columns ilo .. ihi
    const bool rowin = j <= jhi, colin = i >= ilo && i <= ihi;
    SgFace fx{0.f, 0.f, 0.0, 0.0}, fy{0.f, 0.f, 0.0, 0.0};
    if (rowin && i >= ilo - 1 && i <= ihi + 1) fx = smcw_face(umask, p, p + kP, 1, zc, buoy);
    if (colin && j <= jhi + 1) fy = smcw_face(vmask, p, p + kP, nx, zc, buoy);
    sZx[ty][tx + 1] = fx.rz; sRx[ty][tx + 1] = fx.rr;
    sZy[ty + 1][tx] = fy.rz; sRy[ty + 1][tx] = fy.rr;
    if (ty == SG_BY - 1 && tx < 2 * SG_BY) {
        // x faces at columns i0-1 and i0+SG_BX of every row of the tile, all
        // by the last warp (lane 2r + side: row r): one warp's FP64
        // differences instead of one per row
        const int r = tx >> 1, side = tx & 1;
        const int jr = j0 + r;
        const int ii = side == 0 ? i0 - 1 : i0 + SG_BX;
        SgFace f{0.f, 0.f, 0.0, 0.0};
        if (jr <= jhi && ii >= ilo - 1 && ii <= ihi + 1) {
            const long long pp = (long long)jr * nx + ii;
            f = smcw_face(umask, pp, pp + kP, 1, zc, buoy);
        }
        sZx[r][side == 0 ? 0 : SG_BX + 1] = f.rz;
        sRx[r][side == 0 ? 0 : SG_BX + 1] = f.rr;
    }
    if (ty < 2) {  // y faces at rows j0-1 (ty 0) and j0+SG_BY (ty 1) of column i
        const int jj = ty == 0 ? j0 - 1 : j0 + SG_BY;
        SgFace f{0.f, 0.f, 0.0, 0.0};
        if (colin && jj <= jhi + 1) {
            const long long pp = (long long)jj * nx + i;
            f = smcw_face(vmask, pp, pp + kP, nx, zc, buoy);
        }
        sZy[ty == 0 ? 0 : SG_BY + 1][tx] = f.rz;
        sRy[ty == 0 ? 0 : SG_BY + 1][tx] = f.rr;
    }
    __syncthreads();
    if (!rowin || !colin) return;
    const long long q = p + kP;
    const float x = 1.f / 12.f;
    for (int dir = 0; dir < 2; dir++) {
        const int* m = dir ? vmask : umask;
        if (m[p] != 1) continue;
        const long long s = dir ? nx : 1;
        float rZ0, rR0, rZ1, rR1, rZ2, rR2;
        double dzc, dbq;
        if (dir == 0) {
            rZ0 = sZx[ty][tx]; rR0 = sRx[ty][tx];
            rZ1 = sZx[ty][tx + 1]; rR1 = sRx[ty][tx + 1];
            rZ2 = sZx[ty][tx + 2]; rR2 = sRx[ty][tx + 2];
            dzc = fx.dz; dbq = fx.db;
        } else {
            rZ0 = sZy[ty][tx]; rR0 = sRy[ty][tx];
            rZ1 = sZy[ty + 1][tx]; rR1 = sRy[ty + 1][tx];
            rZ2 = sZy[ty + 2][tx]; rR2 = sRy[ty + 2][tx];
            dzc = fy.dz; dbq = fy.db;
        }
        const float dZx0 = smcw_harm_f(rZ0, rZ1), dZx1 = smcw_harm_f(rZ1, rZ2);
        const float dRx0 = smcw_harm_f(rR0, rR1), dRx1 = smcw_harm_f(rR1, rR2);
        const float corr = 0.2f * ((dRx1 - dRx0) * (getm_d2f_approx(dzc) - x * (dZx1 + dZx0)) -
                                   (dZx1 - dZx0) * (getm_d2f_approx(dbq) - x * (dRx1 + dRx0)));
        const double FC = getm_half((buoy[q + s] + buoy[q]) * dzc - getm_f2d(corr));  // 0.5 x, exactly
        // the large, nearly cancelling terms in FP64 (the surface term from
        // the column sweep), the scaling by the mean thickness and the
        // inverse spacing in float
        const double surf = Pw[p + (long long)(nz + dir) * P];
        const float hm = 0.5f * (getm_d2f_approx(h[q]) + getm_d2f_approx(h[q + s]));
        const float idf = getm_d2f_approx(dir ? idyv[p] : idxu[p]);
        double* out = dir ? idpdy : idpdx;
        out[q] = getm_f2d(hm * idf * getm_d2f_approx((Pw[q + s] - Pw[q]) + FC - surf));
    }
}

extern "C" int getm_shchepetkin_mcwilliams_mixed(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                                                 const int* mask, const int* umask, const int* vmask,
                                                 const double* idxu, const double* idyv, const double* h,
                                                 const double* z, const double* zc, const double* buoy,
                                                 double* idpdx, double* idpdy, double* P_work,
                                                 cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || imin < 2 || jmin < 2 || imax + 2 > nx || jmax + 2 > ny || jmax < jmin) return GETM_ERR_ARG;
    if (!mask || !umask || !vmask || !idxu || !idyv || !h || !z || !zc || !buoy || !idpdx || !idpdy || !P_work)
        return GETM_ERR_ARG;
    const unsigned g1 = getm_div_up((long long)nx * (jmax - jmin + 2), 128);
    smcw_column_mixed_kernel<<<g1, 128, 0, stream>>>(nx, ny, nz, imin - 1, imax - 1, jmin - 1, jmax - 1, mask, h, zc,
                                                     buoy, z, P_work);
    GETM_CHECK_LAUNCH();
    dim3 g2(getm_div_up(nx, SG_BX), getm_div_up(jmax - jmin + 1, SG_BY), nz);
    smcw_gradient_mixed_kernel<<<g2, dim3(SG_BX, SG_BY), 0, stream>>>(nx, ny, nz, imin - 1, imax - 1, jmin - 1,
                                                                      jmax - 1, umask, vmask, idxu, idyv, h, zc,
                                                                      buoy, P_work, idpdx, idpdy);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

template <typename T>
static int smcw_impl(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax, const int* mask,
                     const int* umask, const int* vmask, const double* idxu, const double* idyv, const double* h,
                     const double* z, const double* zc, const T* buoy, T* idpdx, T* idpdy, double* P_work,
                     cudaStream_t stream)
{
    // the stencil reaches i+2 / j+2 of the last interior point
    if (nx < 1 || ny < 1 || nz < 1 || imin < 2 || jmin < 2 || imax + 2 > nx || jmax + 2 > ny || jmax < jmin) return GETM_ERR_ARG;
    if (!mask || !umask || !vmask || !idxu || !idyv || !h || !z || !zc || !buoy || !idpdx || !idpdy || !P_work)
        return GETM_ERR_ARG;
    dim3 g1(getm_div_up(nx, 128), jmax - jmin + 2);
    smcw_column_kernel<T><<<g1, 128, 0, stream>>>(nx, ny, nz, imin - 1, imax - 1, jmin - 1, jmax - 1, mask, h, zc, buoy, P_work);
    GETM_CHECK_LAUNCH();
    dim3 g2(getm_div_up(nx, 128), jmax - jmin + 1, nz);
    smcw_gradient_kernel<T><<<g2, 128, 0, stream>>>(nx, ny, nz, imin - 1, imax - 1, jmin - 1, jmax - 1, umask, vmask, idxu, idyv, h, z, zc, buoy, P_work, idpdx, idpdy);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_shchepetkin_mcwilliams(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                                           const int* mask, const int* umask, const int* vmask,
                                           const double* idxu, const double* idyv, const double* h,
                                           const double* z, const double* zc, const double* buoy,
                                           double* idpdx, double* idpdy, double* P_work,
                                           cudaStream_t stream)
{
    return smcw_impl<double>(nx, ny, nz, imin, imax, jmin, jmax, mask, umask, vmask, idxu, idyv, h, z, zc, buoy,
                             idpdx, idpdy, P_work, stream);
}

extern "C" int getm_shchepetkin_mcwilliams_f32(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                                               const int* mask, const int* umask, const int* vmask,
                                               const double* idxu, const double* idyv, const double* h,
                                               const double* z, const double* zc, const float* buoy,
                                               float* idpdx, float* idpdy, double* P_work,
                                               cudaStream_t stream)
{
    return smcw_impl<float>(nx, ny, nz, imin, imax, jmin, jmax, mask, umask, vmask, idxu, idyv, h, z, zc, buoy,
                            idpdx, idpdy, P_work, stream);
}
