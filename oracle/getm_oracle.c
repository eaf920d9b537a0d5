/*
 * CPU oracle: a plain-C restatement of pygetm's Fortran operators on the
 * split-explicit time-step path.  TEST INFRASTRUCTURE ONLY - the CUDA library
 * is compared against it; it is never part of the product path.
 *
 * Every routine cites the reference routine it restates (paths within the
 * BoldingBruggeman/getm project).  Arithmetic is FP64 and follows the Fortran
 * evaluation order operation by operation; build with -ffp-contract=off so no
 * multiply-add is fused (gfortran on generic x86-64 emits none either).
 *
 * Array convention: C order [k][j][i] (i fastest), the layout the Cython layer
 * hands to Fortran (python/_pygetm.pyx:104-114).  A 2D field has nx_*ny_
 * elements.  Index bounds passed in are the Fortran 1-based ones unless stated
 * otherwise, exactly as the reference bind(c) routines receive them.
 *
 * Parity pins: the reference ships no golden vectors and its Fortran cannot be
 * compiled here (no Fortran compiler).  The restatement is pinned against the
 * known-answer and invariant tests of python/tests/ (ported to tests/test_oracle_*.py).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define IDX2(i, j) ((size_t)(j) * (size_t)nx_ + (size_t)(i))
#define IDX3(i, j, k) (((size_t)(k) * (size_t)ny_ + (size_t)(j)) * (size_t)nx_ + (size_t)(i))

static const double RHO0 = 1025.0;  /* python/src/wrapper.F90:11 */
static const double KAPPA = 0.4;    /* python/src/wrapper.F90:12 */
static const double G = 9.81;       /* python/src/wrapper.F90:13 */

static double dmin2(double a, double b) { return a < b ? a : b; }
static double dmax2(double a, double b) { return a > b ? a : b; }

/* ------------------------------------------------------------------------ */
/* TVD limiters: src/operators/advection_schemes/limiters.h:1-44             */
/* scheme codes follow src/operators/advection.F90:22-30                     */
/* ------------------------------------------------------------------------ */
double oracle_limiter(int scheme, double ratio, double cfl)
{
    double limiter = 0.0;
    switch (scheme) {
    case 1: { /* HSIMT limiters.h:2-11 */
        double kappa = 1 - cfl;
        double x = 0.25 * (kappa - 1.0 / 3.0 / kappa);
        limiter = (0.5 + x) + (0.5 - x) * ratio;
        limiter = dmax2(0.0, limiter);
        limiter = dmin2(dmin2(2.0 * ratio, limiter), 2.0);
        break;
    }
    case 2: /* MUSCL limiters.h:13-17 */
        limiter = dmin2(dmin2(2 * ratio, 0.5 * (1 + ratio)), 2.0);
        break;
    case 3: { /* P2_PDM limiters.h:19-26 */
        double x = 1.0 / 6.0 * (1.0 - 2.0 * cfl);
        limiter = (0.5 + x) + (0.5 - x) * ratio;
        limiter = dmin2(dmin2(2.0 * ratio / (cfl + 1.e-10), limiter), 2.0 / (1.0 - cfl));
        break;
    }
    case 4: /* SPLMAX13 limiters.h:28-32 */
        limiter = dmin2(dmin2(2.0 * ratio, 1.0 / 3.0 * dmax2(1.0 + 2.0 * ratio, 2.0 + ratio)), 2.0);
        break;
    case 5: /* SUPERBEE limiters.h:34-38 */
        limiter = dmax2(dmin2(2.0 * ratio, 1.0), dmin2(ratio, 2.0));
        break;
    default: /* UPSTREAM limiters.h:40-44 */
        limiter = 0.0;
        break;
    }
    return limiter;
}

/* ------------------------------------------------------------------------ */
/* Directional horizontal advection of one layer.                            */
/* u-direction: src/operators/advection_schemes/advection.F90.template:23-121 */
/* v-direction: same template :123-221.                                      */
/* imin..imax, jmin..jmax are Fortran interior bounds; arrays span           */
/* imin-halox..imax+halox, jmin-haloy..jmax+haloy.                           */
/* ------------------------------------------------------------------------ */
static void advect_layer(int direction, int scheme, int imin, int imax, int jmin, int jmax,
                         int halox, int haloy, const int *umask, const double *idxu,
                         const double *dyu, const double *hu, const double *u,
                         const int *tmask, const double *iA, int apply_diffusion,
                         const double *Ah, double dt, double *h, double *f,
                         double *flux, double *QU)
{
    const int nx_ = imax - imin + 1 + 2 * halox;
    const int ny_ = jmax - jmin + 1 + 2 * haloy;
    /* C index of Fortran (i, j) */
#define C2(i, j) IDX2((i) - (imin - halox), (j) - (jmin - haloy))
    /* stride of the advected direction (u: +1 in i; v: +1 in j) */
    const size_t s = (direction == 1) ? 1 : (size_t)nx_;
    const int fi0 = (direction == 1) ? imin - 1 : imin;
    const int fj0 = (direction == 1) ? jmin : jmin - 1;
    for (int j = fj0; j <= jmax; j++) {
        for (int i = fi0; i <= imax; i++) {
            size_t p = C2(i, j);
            if (umask[p] == 1 || umask[p] == 2) {
                QU[p] = u[p] * hu[p] * dyu[p];
                double cfl = fabs(u[p] * dt * idxu[p]);
                double fu, fuu, fd;
                if (u[p] > 0) {
                    fu = f[p];
                    fuu = fu;
                    if (umask[p - s] == 1 || umask[p - s] == 2) fuu = f[p - s];
                    fd = f[p + s];
                } else {
                    fu = f[p + s];
                    fuu = fu;
                    if (umask[p + s] == 1 || umask[p + s] == 2) fuu = f[p + 2 * s];
                    fd = f[p];
                }
                double deltaf = fd - fu;
                double deltafu = fu - fuu;
                if (deltaf * deltafu > 0) {
                    double ratio = deltafu / deltaf;
                    double limiter = oracle_limiter(scheme, ratio, cfl);
                    fu = fu + 0.5 * limiter * (1 - cfl) * deltaf;
                }
                flux[p] = QU[p] * fu;
            } else {
                QU[p] = 0.0;
                flux[p] = 0.0;
            }
        }
    }
    if (apply_diffusion) { /* template :97-105 / :197-205 */
        for (int j = fj0; j <= jmax; j++) {
            for (int i = fi0; i <= imax; i++) {
                size_t p = C2(i, j);
                if (umask[p] == 1 || umask[p] == 2)
                    flux[p] = flux[p] - Ah[p] * hu[p] * (f[p + s] - f[p]) * idxu[p] * dyu[p];
            }
        }
    }
    for (int j = jmin; j <= jmax; j++) { /* template :107-116 / :207-216 */
        for (int i = imin; i <= imax; i++) {
            size_t p = C2(i, j);
            if (tmask[p] == 1) {
                double hfo = h[p] * f[p];
                h[p] = h[p] - dt * (QU[p] - QU[p - s]) * iA[p];
                double advn = (flux[p] - flux[p - s]) * iA[p];
                f[p] = (hfo - dt * advn) / h[p];
            }
        }
    }
#undef C2
}

/* python/src/wrapper.F90:213-254 advection_uv_calculate: loop over nk layers.
 * direction 1: u-grid metrics (mask, idx, dy); direction 2: v-grid metrics
 * (mask, dx, idy) - passed here as (umask, idxu=dx-or-idx, dyu=...) in the
 * template's own argument order.  Ah == NULL means no horizontal diffusion.  */
void oracle_advection_uv_calculate(int direction, int nk, int scheme, int imin, int imax,
                                   int jmin, int jmax, int halox, int haloy,
                                   const int *umask, const double *m1, const double *m2,
                                   const double *u, const double *Ah, double timestep,
                                   double *h, const double *hu, double *var,
                                   const int *tmask, const double *iA)
{
    const size_t n2 = (size_t)(imax - imin + 1 + 2 * halox) * (size_t)(jmax - jmin + 1 + 2 * haloy);
    /* layers are independent (wrapper.F90:242-252): threads take whole layers */
#pragma omp parallel
    {
        double *flux = (double *)calloc(n2, sizeof(double));
        double *QU = (double *)calloc(n2, sizeof(double));
#pragma omp for schedule(static)
        for (int k = 0; k < nk; k++) {
            /* u2d receives (umask, idxu, dyu); v2d receives (vmask, dxv, idyv) and
             * uses dxv in the transport and idyv in the cfl (template :164-165). */
            const double *idx_ = (direction == 1) ? m1 : m2;
            const double *dy_ = (direction == 1) ? m2 : m1;
            advect_layer(direction, scheme, imin, imax, jmin, jmax, halox, haloy, umask, idx_, dy_,
                         hu + k * n2, u + k * n2, tmask, iA, Ah != NULL, Ah ? Ah : u, timestep,
                         h + k * n2, var + k * n2, flux, QU);
        }
        free(flux);
        free(QU);
    }
}

/* ------------------------------------------------------------------------ */
/* Vertical advection with adaptive sub-stepping:                            */
/* src/operators/advection_schemes/advection.F90.template:223-374            */
/* w, w_var have kmax+1 levels (interfaces 0..kmax); h, f have kmax levels.  */
/* Returns the largest iteration count used (for itersmax reporting).        */
/* ------------------------------------------------------------------------ */
int oracle_advection_w_calculate(int scheme, int imin, int imax, int jmin, int jmax, int kmax,
                                 int halox, int haloy, const double *w, const double *w_var,
                                 const int *tmask, double dt, double *h, double *f)
{
    const int itersmax = 200;
    const int nx_ = imax - imin + 1 + 2 * halox;
    const int ny_ = jmax - jmin + 1 + 2 * haloy;
    int maxiters = 0;
    /* Fortran level k of h/f (1..kmax) -> C plane k-1; w level k (0..kmax) -> plane k */
#define HF(i, j, k) IDX3((i) - (imin - halox), (j) - (jmin - haloy), (k) - 1)
#define WW(i, j, k) IDX3((i) - (imin - halox), (j) - (jmin - haloy), (k))
#pragma omp parallel reduction(max : maxiters)
    {
    double *flux = (double *)calloc((size_t)kmax + 1, sizeof(double));
    double *cfl0 = (double *)calloc((size_t)kmax + 1, sizeof(double));
    double *cfls = (double *)calloc((size_t)kmax + 1, sizeof(double));
    double *haux = (double *)calloc((size_t)kmax + 1, sizeof(double));
    double *faux = (double *)calloc((size_t)kmax + 1, sizeof(double));
    flux[0] = 0.0;
    flux[kmax] = 0.0;
#pragma omp for schedule(dynamic, 4)
    for (int j = jmin; j <= jmax; j++) {
        for (int i = imin; i <= imax; i++) {
            if (tmask[IDX2(i - (imin - halox), j - (jmin - haloy))] != 1) continue;
            for (int k = 1; k <= kmax - 1; k++)
                cfl0[k] = fabs(w_var[WW(i, j, k)]) * dt / dmin2(h[HF(i, j, k)], h[HF(i, j, k + 1)]);
            int iters = 1;
            double itersm1 = 1.0;
            double dtk = dt;
            int it = 1;
            while (it <= iters) {
                if (it == 1) {
                    for (int k = 1; k <= kmax; k++) {
                        haux[k] = h[HF(i, j, k)];
                        faux[k] = f[HF(i, j, k)];
                    }
                    for (int k = 1; k <= kmax - 1; k++) cfls[k] = cfl0[k];
                } else {
                    for (int k = 1; k <= kmax - 1; k++)
                        cfls[k] = fabs(w_var[WW(i, j, k)]) * dt / dmin2(haux[k], haux[k + 1]);
                }
                if (iters < itersmax) {
                    /* MAXVAL over an empty range (kmax == 1) gives -HUGE -> iters_new = 1 */
                    int iters_new = 1;
                    if (kmax > 1) {
                        double cfl = cfls[1];
                        for (int k = 2; k <= kmax - 1; k++)
                            if (cfls[k] > cfl) cfl = cfls[k];
                        double c = ceil(cfl);
                        iters_new = c > 1.0 ? (c > 1e9 ? 1000000000 : (int)c) : 1;
                    }
                    if (iters_new > iters) {
                        iters = iters_new > itersmax ? itersmax : iters_new;
                        itersm1 = 1.0 / iters;
                        dtk = dt * itersm1;
                        if (it > 1) {
                            it = 1;
                            continue;
                        }
                    }
                }
                for (int k = 1; k <= kmax - 1; k++) {
                    double cfl = cfls[k] * itersm1;
                    double wv = w_var[WW(i, j, k)];
                    double fu, fuu, fd;
                    if (wv > 0) {
                        fu = faux[k];
                        fuu = (k > 1) ? faux[k - 1] : fu;
                        fd = faux[k + 1];
                    } else {
                        fu = faux[k + 1];
                        fuu = (k < kmax - 1) ? faux[k + 2] : fu;
                        fd = faux[k];
                    }
                    double deltaf = fd - fu;
                    double deltafu = fu - fuu;
                    if (deltaf * deltafu > 0) {
                        double ratio = deltafu / deltaf;
                        double limiter = oracle_limiter(scheme, ratio, cfl);
                        fu = fu + 0.5 * limiter * (1 - cfl) * deltaf;
                    }
                    flux[k] = wv * fu;
                }
                const int last = (it == iters);
                for (int k = 1; k <= kmax; k++) {
                    double hfo = haux[k] * faux[k];
                    double hnew = haux[k] - dtk * (w[WW(i, j, k)] - w[WW(i, j, k - 1)]);
                    double advn = flux[k] - flux[k - 1];
                    double fnew = (hfo - dtk * advn) / hnew;
                    if (last) {
                        h[HF(i, j, k)] = hnew;
                        f[HF(i, j, k)] = fnew;
                    } else {
                        haux[k] = hnew;
                        faux[k] = fnew;
                    }
                }
                it = it + 1;
            }
            if (iters > maxiters) maxiters = iters;
        }
    }
    free(flux);
    free(cfl0);
    free(cfls);
    free(haux);
    free(faux);
    }
#undef HF
#undef WW
    return maxiters;
}

/* ------------------------------------------------------------------------ */
/* Implicit vertical diffusion: src/operators/diffusion.F90:135-314 reached  */
/* through python/src/wrapper.F90:149-186.  auxo/auxn are caller-provided    */
/* work arrays of nx_*ny_*nz (only levels 0..nz-2 used, = Fortran 1..nz-1).  */
/* nuh has nz+1 interface levels; levels 1..nz-1 are read (wrapper.F90:160). */
/* ------------------------------------------------------------------------ */
void oracle_vertical_diffusion_prepare(int nx_, int ny_, int nz, double molecular,
                                       const double *nuh, double dt, double cnpar,
                                       const int *mask, const double *dzo, const double *dzn,
                                       double *auxo, double *auxn)
{
    (void)mask;
    if (nz == 1) return; /* diffusion.F90:155 */
    /* diffusion.F90:163-171: all i, j including halos; Fortran k = kmin..kmax-1 */
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nz - 1; k++) {
        for (int j = 0; j < ny_; j++) {
            for (int i = 0; i < nx_; i++) {
                double x = 2.0 * dt * (nuh[IDX3(i, j, k)] + molecular);
                auxo[IDX3(i, j, k - 1)] = (1.0 - cnpar) * x / (dzo[IDX3(i, j, k)] + dzo[IDX3(i, j, k - 1)]);
                auxn[IDX3(i, j, k - 1)] = cnpar * x / (dzn[IDX3(i, j, k)] + dzn[IDX3(i, j, k - 1)]);
            }
        }
    }
    /* a1 = -auxn(k-1), a3 = -auxn(k) (diffusion.F90:173-198) are formed in apply. */
}

void oracle_vertical_diffusion_apply(int nx_, int ny_, int nz, const int *mask,
                                     const double *dzo, const double *dzn, double *var,
                                     const double *ea2, const double *ea4,
                                     const double *auxo, const double *auxn)
{
    if (nz == 1) { /* diffusion.F90:224-231: every point, mask not consulted */
        for (size_t p = 0; p < (size_t)nx_ * ny_; p++) {
            double a4 = dzo[p] * var[p];
            double a2 = dzn[p];
            if (ea4) a4 = a4 + ea4[p];
            if (ea2) a2 = a2 - ea2[p];
            var[p] = a4 / a2;
        }
        return;
    }
    const int kmin = 0, kmax = nz - 1; /* C levels; Fortran kmin=1..kmax=nz */
#pragma omp parallel
    {
    double *a1 = (double *)malloc(sizeof(double) * nz);
    double *a2 = (double *)malloc(sizeof(double) * nz);
    double *a3 = (double *)malloc(sizeof(double) * nz);
    double *a4 = (double *)malloc(sizeof(double) * nz);
    double *ru = (double *)malloc(sizeof(double) * nz);
    double *qu = (double *)malloc(sizeof(double) * nz);
#pragma omp for schedule(static)
    for (int j = 0; j < ny_; j++) {
        for (int i = 0; i < nx_; i++) {
            if (mask[IDX2(i, j)] != 1) continue;
#define V(k) var[IDX3(i, j, k)]
#define AO(k) auxo[IDX3(i, j, k)]
#define AN(k) auxn[IDX3(i, j, k)]
            /* surface layer diffusion.F90:238-245 (and a1 from :174-179) */
            int k = kmax;
            a1[k] = -AN(k - 1);
            a2[k] = dzn[IDX3(i, j, k)] + AN(k - 1);
            a4[k] = V(k) * dzo[IDX3(i, j, k)] + (V(k - 1) - V(k)) * AO(k - 1);
            /* inner layers :247-258 (and a1/a3 from :181-190) */
            for (k = kmin + 1; k <= kmax - 1; k++) {
                a3[k] = -AN(k);
                a1[k] = -AN(k - 1);
                a2[k] = dzn[IDX3(i, j, k)] + AN(k) + AN(k - 1);
                a4[k] = V(k) * dzo[IDX3(i, j, k)] + (V(k + 1) - V(k)) * AO(k) + (V(k - 1) - V(k)) * AO(k - 1);
            }
            /* bottom layer :260-267 (and a3 from :192-198) */
            k = kmin;
            a3[k] = -AN(k);
            a2[k] = dzn[IDX3(i, j, k)] + AN(k);
            a4[k] = V(k) * dzo[IDX3(i, j, k)] + (V(k + 1) - V(k)) * AO(k);
            for (k = kmin; k <= kmax; k++) { /* :269-270 */
                if (ea2) a2[k] = a2[k] - ea2[IDX3(i, j, k)];
                if (ea4) a4[k] = a4[k] + ea4[IDX3(i, j, k)];
            }
            /* Thomas algorithm :283-307 */
            ru[kmax] = a1[kmax] / a2[kmax];
            qu[kmax] = a4[kmax] / a2[kmax];
            for (k = kmax - 1; k >= kmin + 1; k--) {
                ru[k] = a1[k] / (a2[k] - a3[k] * ru[k + 1]);
                qu[k] = (a4[k] - a3[k] * qu[k + 1]) / (a2[k] - a3[k] * ru[k + 1]);
            }
            qu[kmin] = (a4[kmin] - a3[kmin] * qu[kmin + 1]) / (a2[kmin] - a3[kmin] * ru[kmin + 1]);
            V(kmin) = qu[kmin];
            for (k = kmin + 1; k <= kmax; k++) V(k) = qu[k] - ru[k] * V(k - 1);
#undef V
#undef AO
#undef AN
        }
    }
    free(a1); free(a2); free(a3); free(a4); free(ru); free(qu);
    }
}

/* ------------------------------------------------------------------------ */
/* Staggered interpolation: python/src/interpolation.F90:9-72                */
/* ------------------------------------------------------------------------ */
void oracle_grid_interp_x(int nx_, int ny_, int nz, const double *source, double *target, int ioffset)
{
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny_; j++)
            for (int i = 0; i < nx_ - 1; i++)
                target[IDX3(i + ioffset, j, k)] = 0.5 * (source[IDX3(i, j, k)] + source[IDX3(i + 1, j, k)]);
}

void oracle_grid_interp_y(int nx_, int ny_, int nz, const double *source, double *target, int joffset)
{
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny_ - 1; j++)
            for (int i = 0; i < nx_; i++)
                target[IDX3(i, j + joffset, k)] = 0.5 * (source[IDX3(i, j, k)] + source[IDX3(i, j + 1, k)]);
}

void oracle_grid_interp_z(int nx_, int ny_, int nz1, int nz2, const double *source, double *target, int koffset)
{
    (void)nz2;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz1 - 1; k++)
        for (int j = 0; j < ny_; j++)
            for (int i = 0; i < nx_; i++)
                target[IDX3(i, j, k + koffset)] = 0.5 * (source[IDX3(i, j, k)] + source[IDX3(i, j, k + 1)]);
}

void oracle_grid_interp_xy(int nx1, int ny1, int nx2, int ny2, int nz, const double *source,
                           double *target, int ioffset, int joffset)
{
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny1 - 1; j++)
            for (int i = 0; i < nx1 - 1; i++) {
                size_t s = ((size_t)k * ny1 + j) * nx1 + i;
                size_t t = ((size_t)k * ny2 + j + joffset) * nx2 + i + ioffset;
                target[t] = 0.25 * (source[s] + source[s + 1] + source[s + nx1] + source[s + nx1 + 1]);
            }
}

/* ------------------------------------------------------------------------ */
/* python/src/wrapper.F90 2D/column utilities                                */
/* ------------------------------------------------------------------------ */
/* wrapper.F90:437-445 */
void oracle_elevation2depth(int n, const double *z, const double *H, double Dmin, const int *mask, double *D)
{
    for (int p = 0; p < n; p++)
        if (mask[p] != 0) D[p] = dmax2(H[p] + z[p], Dmin);
}

/* wrapper.F90:428-435 */
void oracle_alpha(int n, const double *D, double Dmin, double Dcrit, const int *mask, double *alpha)
{
    for (int p = 0; p < n; p++)
        if (mask[p] != 0) alpha[p] = dmax2(0.0, dmin2(1.0, (D[p] - Dmin) / (Dcrit - Dmin)));
}

/* wrapper.F90:409-426 */
void oracle_thickness2vertical_coordinates(int nx_, int ny_, int nz, const int *mask,
                                           const double *bottom_depth, const double *h,
                                           double *zc, double *zf)
{
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny_; j++)
        for (int i = 0; i < nx_; i++) {
            size_t p = IDX2(i, j);
            if (mask[p] == 0) continue;
            zc[IDX3(i, j, 0)] = -bottom_depth[p] + 0.5 * h[IDX3(i, j, 0)];
            for (int k = 1; k < nz; k++)
                zc[IDX3(i, j, k)] = zc[IDX3(i, j, k - 1)] + 0.5 * (h[IDX3(i, j, k - 1)] + h[IDX3(i, j, k)]);
            zf[IDX3(i, j, 0)] = -bottom_depth[p];
            for (int k = 1; k <= nz; k++)
                zf[IDX3(i, j, k)] = zf[IDX3(i, j, k - 1)] + h[IDX3(i, j, k - 1)];
        }
}

/* wrapper.F90:395-407 (istart..jstop unused by the reference routine too) */
void oracle_thickness2center_depth(int nx_, int ny_, int nz, const int *mask, const double *h, double *out)
{
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny_; j++)
        for (int i = 0; i < nx_; i++) {
            if (mask[IDX2(i, j)] == 0) continue;
            out[IDX3(i, j, nz - 1)] = 0.5 * h[IDX3(i, j, nz - 1)];
            for (int k = nz - 2; k >= 0; k--)
                out[IDX3(i, j, k)] = out[IDX3(i, j, k + 1)] + 0.5 * (h[IDX3(i, j, k)] + h[IDX3(i, j, k + 1)]);
        }
}

/* wrapper.F90:496-523 */
void oracle_advance_surface_elevation(int nx_, int ny_, int halox, int haloy, const int *mask,
                                      const double *dyu, const double *dxv, const double *iarea,
                                      double *z, const double *U, const double *V,
                                      const double *fwf, double dt)
{
    for (int j = haloy; j < ny_ - haloy; j++)
        for (int i = halox; i < nx_ - halox; i++) {
            size_t p = IDX2(i, j);
            if (mask[p] == 1)
                z[p] = z[p] + dt * ((U[p - 1] * dyu[p - 1] - U[p] * dyu[p] + V[p - nx_] * dxv[p - nx_] - V[p] * dxv[p]) * iarea[p] + fwf[p]);
        }
}

/* wrapper.F90:525-565 (imin..jmax Fortran 1-based) */
void oracle_surface_pressure_gradient(int nx_, int ny_, int imin, int imax, int jmin, int jmax,
                                      const int *umask, const int *vmask, const double *idxu,
                                      const double *idyv, const double *z, const double *sp,
                                      const double *H, const double *D, double Dmin,
                                      double *dpdx, double *dpdy)
{
    const double gammai = 1.0 / (G * RHO0);
    (void)ny_;
    for (int j = jmin - 1; j <= jmax - 1; j++)
        for (int i = imin - 1; i <= imax - 1; i++) {
            size_t p = IDX2(i, j);
            if (umask[p] == 1) {
                double zp = dmax2(z[p + 1], -H[p] + dmin2(Dmin, D[p + 1]));
                double zm = dmax2(z[p], -H[p + 1] + dmin2(Dmin, D[p]));
                dpdx[p] = (zp - zm + (sp[p + 1] - sp[p]) * gammai) * idxu[p];
            }
        }
    for (int j = jmin - 1; j <= jmax - 1; j++)
        for (int i = imin - 1; i <= imax - 1; i++) {
            size_t p = IDX2(i, j);
            if (vmask[p] == 1) {
                double zp = dmax2(z[p + nx_], -H[p] + dmin2(Dmin, D[p + nx_]));
                double zm = dmax2(z[p], -H[p + nx_] + dmin2(Dmin, D[p]));
                dpdy[p] = (zp - zm + (sp[p + nx_] - sp[p]) * gammai) * idyv[p];
            }
        }
}

/* wrapper.F90:275-393 c_momentum_diffusion (one layer per k).
 * Grid bounds: interior C ranges [ilo, ihi] x [jlo, jhi] of the U grid; all six
 * grids share the same array extents (nx_, ny_) and interior, as pygetm creates
 * them (python/pygetm/domain.py:699-725).                                   */
void oracle_momentum_diffusion(int nx_, int ny_, int nk, int halox, int haloy,
                               const int *umask, const double *uiarea,
                               const int *vmask, const double *viarea,
                               const int *uumask, const double *uudy, const double *uuidx,
                               const int *uvmask, const double *uvdx, const double *uvidx, const double *uvidy,
                               const int *vumask, const double *vudy, const double *vuidx, const double *vuidy,
                               const int *vvmask, const double *vvdx, const double *vvidy,
                               const double *huu, const double *huv, const double *hvu, const double *hvv,
                               const double *u, const double *v, double Am0,
                               double *diffu, double *diffv)
{
    const int ilo = halox, ihi = nx_ - halox - 1, jlo = haloy, jhi = ny_ - haloy - 1;
    const size_t n2 = (size_t)nx_ * ny_;
    double *flux = (double *)calloc(n2, sizeof(double));
    for (int k = 0; k < nk; k++) {
        const double *uk = u + k * n2, *vk = v + k * n2;
        const double *huuk = huu + k * n2, *huvk = huv + k * n2, *hvuk = hvu + k * n2, *hvvk = hvv + k * n2;
        double *du = diffu + k * n2, *dv = diffv + k * n2;
        /* :323-339 */
        for (int j = jlo; j <= jhi; j++)
            for (int i = ilo - 1; i <= ihi; i++) {
                size_t p = IDX2(i, j);
                flux[p] = 0.0;
                if (uumask[p] != 0)
                    flux[p] = 2.0 * Am0 * uudy[p] * huuk[p] * (uk[p + 1] - uk[p]) * uuidx[p];
            }
        for (int j = jlo; j <= jhi; j++)
            for (int i = ilo; i <= ihi; i++) {
                size_t p = IDX2(i, j);
                du[p] = 0.0;
                if (umask[p] == 1) du[p] = (flux[p] - flux[p - 1]) * uiarea[p];
            }
        /* :341-356 */
        for (int j = jlo - 1; j <= jhi; j++)
            for (int i = ilo; i <= ihi; i++) {
                size_t p = IDX2(i, j);
                flux[p] = 0.0;
                if (uvmask[p] != 0)
                    flux[p] = Am0 * uvdx[p] * huvk[p] * ((uk[p + nx_] - uk[p]) * uvidy[p] + (vk[p + 1] - vk[p]) * uvidx[p]);
            }
        for (int j = jlo; j <= jhi; j++)
            for (int i = ilo; i <= ihi; i++) {
                size_t p = IDX2(i, j);
                if (umask[p] == 1 || umask[p] == 2) du[p] = du[p] + (flux[p] - flux[p - nx_]) * uiarea[p];
            }
        /* :358-374 */
        for (int j = jlo; j <= jhi; j++)
            for (int i = ilo - 1; i <= ihi; i++) {
                size_t p = IDX2(i, j);
                flux[p] = 0.0;
                if (vumask[p] != 0)
                    flux[p] = Am0 * vudy[p] * hvuk[p] * ((uk[p + nx_] - uk[p]) * vuidy[p] + (vk[p + 1] - vk[p]) * vuidx[p]);
            }
        for (int j = jlo; j <= jhi; j++)
            for (int i = ilo; i <= ihi; i++) {
                size_t p = IDX2(i, j);
                dv[p] = 0.0;
                if (vmask[p] == 1) dv[p] = (flux[p] - flux[p - 1]) * viarea[p];
            }
        /* :376-391 */
        for (int j = jlo - 1; j <= jhi; j++)
            for (int i = ilo; i <= ihi; i++) {
                size_t p = IDX2(i, j);
                flux[p] = 0.0;
                if (vvmask[p] != 0)
                    flux[p] = 2.0 * Am0 * vvdx[p] * hvvk[p] * (vk[p + nx_] - vk[p]) * vvidy[p];
            }
        for (int j = jlo; j <= jhi; j++)
            for (int i = ilo; i <= ihi; i++) {
                size_t p = IDX2(i, j);
                if (vmask[p] == 1) dv[p] = dv[p] + (flux[p] - flux[p - nx_]) * viarea[p];
            }
    }
    free(flux);
}

/* ------------------------------------------------------------------------ */
/* python/src/momentum.F90                                                   */
/* ------------------------------------------------------------------------ */
/* momentum.F90:12-77 (imin..jmax Fortran interior bounds, 1-based) */
void oracle_horizontal_diffusion(int imin, int imax, int jmin, int jmax, int halox, int haloy,
                                 const int *umask, const int *vmask, const double *idxu,
                                 const double *dyu, const double *idyv, const double *dxv,
                                 const double *Ah_u, const double *Ah_v, const int *tmask,
                                 const double *iA, double dt, const double *f, double *df)
{
    const int nx_ = imax - imin + 1 + 2 * halox;
    const int ny_ = jmax - jmin + 1 + 2 * haloy;
    double *uflux = (double *)calloc((size_t)nx_ * ny_, sizeof(double));
    double *vflux = (double *)calloc((size_t)nx_ * ny_, sizeof(double));
#define C2(i, j) IDX2((i) - (imin - halox), (j) - (jmin - haloy))
    for (int j = jmin; j <= jmax; j++)
        for (int i = imin - 1; i <= imax; i++) {
            size_t p = C2(i, j);
            uflux[p] = (umask[p] == 1) ? Ah_u[p] * (f[p + 1] - f[p]) * idxu[p] * dyu[p] : 0.0;
        }
    for (int j = jmin - 1; j <= jmax; j++)
        for (int i = imin; i <= imax; i++) {
            size_t p = C2(i, j);
            vflux[p] = (vmask[p] == 1) ? Ah_v[p] * (f[p + nx_] - f[p]) * idyv[p] * dxv[p] : 0.0;
        }
    for (int j = jmin; j <= jmax; j++)
        for (int i = imin; i <= imax; i++) {
            size_t p = C2(i, j);
            if (tmask[p] == 1)
                df[p] = dt * (uflux[p] - uflux[p - 1] + vflux[p] - vflux[p - nx_]) * iA[p];
        }
#undef C2
    free(uflux);
    free(vflux);
}

/* momentum.F90:79-101 */
void oracle_bottom_friction(int nx_, int ny_, const int *mask, const double *u, const double *v,
                            const double *D, double *z0b, const double *z0b_min, double avmmol,
                            double *ru, int iterate)
{
    for (size_t p = 0; p < (size_t)nx_ * ny_; p++) {
        if (mask[p] != 1) continue;
        double sqrtcd = KAPPA / log(1.0 + 0.5 * D[p] / z0b[p]);
        if (iterate != 0) {
            z0b[p] = dmin2(D[p], z0b_min[p] + 0.1 * avmmol / dmax2(avmmol, sqrtcd * sqrt(u[p] * u[p] + v[p] * v[p])));
            sqrtcd = KAPPA / log(1.0 + 0.5 * D[p] / z0b[p]);
        }
        ru[p] = sqrtcd * sqrtcd * sqrt(u[p] * u[p] + v[p] * v[p]);
    }
}

/* momentum.F90:103-145 (rows haloy..ny_-haloy-1, all i, mask not consulted) */
void oracle_collect_3d_momentum_sources(int nx_, int ny_, int nz, int halox, int haloy,
                                        const int *mask, const double *alpha, const double *ho,
                                        const double *hn, const double *dp, const double *cor,
                                        const double *adv, const double *diff, const double *idp,
                                        const double *taus, const double *rr, double dt,
                                        double *ea2, double *ea4)
{
    (void)mask;
    (void)halox;
    const double rho0i = 1.0 / RHO0;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; k++)
        for (int j = haloy; j < ny_ - haloy; j++)
            for (int i = 0; i < nx_; i++) {
                size_t p = IDX2(i, j), q = IDX3(i, j, k);
                ea4[q] = dt * (-0.5 * (ho[q] + hn[q]) * G * dp[p] + alpha[p] * (cor[q] + adv[q] + diff[q] + idp[q]));
            }
    for (int j = haloy; j < ny_ - haloy; j++)
        for (int i = 0; i < nx_; i++) {
            size_t p = IDX2(i, j);
            ea4[IDX3(i, j, nz - 1)] = ea4[IDX3(i, j, nz - 1)] + dt * alpha[p] * taus[p] * rho0i;
            ea2[IDX3(i, j, 0)] = -dt * rr[p];
        }
}

/* momentum.F90:147-189 */
void oracle_advance_2d_transport(int nx_, int ny_, int halox, int haloy, const int *mask,
                                 const double *alpha, const double *D, const double *dp,
                                 const double *taus, const double *cor, const double *adv,
                                 const double *diff, const double *damp, const double *SA,
                                 const double *SB, const double *SD, const double *SF,
                                 const double *r, double dt, double *U)
{
    const double rho0i = 1.0 / RHO0;
    for (int j = haloy; j < ny_ - haloy; j++)
        for (int i = halox; i < nx_ - halox; i++) {
            size_t p = IDX2(i, j);
            if (mask[p] != 1) continue;
            double Slr = (U[p] > 0.0) ? dmin2(SF[p], 0.0) : dmax2(SF[p], 0.0);
            U[p] = (U[p] + dt * (-G * D[p] * dp[p] + alpha[p] * (taus[p] * rho0i + cor[p] + adv[p] + diff[p] + damp[p] + SA[p] + SB[p] + SD[p] + Slr))) / (1.0 + dt * r[p] / D[p]);
        }
}

/* momentum.F90:191-216 (imin..jmax Fortran 1-based as passed by pyx:454) */
void oracle_w_momentum_3d(int nx_, int ny_, int nz, int imin, int imax, int jmin, int jmax,
                          const int *mask, const double *dyu, const double *dxv,
                          const double *iarea, const double *ho, const double *hn,
                          const double *pk, const double *qk, double dt, double *w)
{
    const double idt = 1.0 / dt;
    /* w has nz+1 levels (0..nz); h/pk/qk level k (1..nz) is C plane k-1 */
#pragma omp parallel for schedule(static)
    for (int j = jmin - 1; j <= jmax - 1; j++)
        for (int k = 1; k <= nz - 1; k++)
            for (int i = imin - 1; i <= imax - 1; i++) {
                size_t p = IDX2(i, j);
                if (mask[p] != 1) continue;
                size_t q = IDX3(i, j, k - 1);
                w[IDX3(i, j, k)] = w[IDX3(i, j, k - 1)] - (hn[q] - ho[q]) * idt
                    - (pk[q] * dyu[p] - pk[q - 1] * dyu[p - 1] + qk[q] * dxv[p] - qk[q - nx_] * dxv[p - nx_]) * iarea[p];
            }
}

/* momentum.F90:218-241 */
void oracle_shear_frequency(int nx_, int ny_, int nz, int imin, int imax, int jmin, int jmax,
                            const int *mask, const double *hu, const double *hv,
                            const double *uk, const double *vk, double *SS)
{
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nz - 1; k++)
        for (int j = jmin - 1; j <= jmax - 1; j++)
            for (int i = imin - 1; i <= imax - 1; i++) {
                size_t p = IDX2(i, j);
                if (mask[p] <= 0) continue;
                size_t a = IDX3(i, j, k - 1), b = IDX3(i, j, k); /* Fortran k, k+1 */
                double t1 = (uk[b] - uk[a]) / (0.5 * (hu[b] + hu[a]));
                double t2 = (uk[b - 1] - uk[a - 1]) / (0.5 * (hu[b - 1] + hu[a - 1]));
                double t3 = (vk[b] - vk[a]) / (0.5 * (hv[b] + hv[a]));
                double t4 = (vk[b - nx_] - vk[a - nx_]) / (0.5 * (hv[b - nx_] + hv[a - nx_]));
                SS[IDX3(i, j, k)] = 0.5 * (t1 * t1 + t2 * t2 + t3 * t3 + t4 * t4);
            }
}

/* momentum.F90:244-268: interfaces k = 1..nz-1 (the layers Fortran k, k+1 are
   0-based k-1, k; interface k is 0-based k), left-to-right evaluation */
void oracle_shear_frequency2(int nx_, int ny_, int nz, int imin, int imax, int jmin, int jmax, const int *mask,
                             const double *h, const double *hu, const double *hv, const double *uk,
                             const double *vk, const double *num, double *SS)
{
    for (int k = 1; k <= nz - 1; k++)
        for (int j = jmin - 1; j <= jmax - 1; j++)
            for (int i = imin - 1; i <= imax - 1; i++) {
                size_t p = IDX2(i, j);
                if (mask[p] <= 0) continue;
                size_t a = IDX3(i, j, k - 1), b = IDX3(i, j, k), q = IDX3(i, j, k);
                double due = uk[b] - uk[a], duw = uk[b - 1] - uk[a - 1];
                double dvn = vk[b] - vk[a], dvs = vk[b - nx_] - vk[a - nx_];
                double s = due * due / (hu[b] + hu[a]) * (num[q] + num[q + 1])
                           + duw * duw / (hu[b - 1] + hu[a - 1]) * (num[q - 1] + num[q])
                           + dvn * dvn / (hv[b] + hv[a]) * (num[q] + num[q + nx_])
                           + dvs * dvs / (hv[b - nx_] + hv[a - nx_]) * (num[q - nx_] + num[q]);
                SS[q] = 0.5 * s / (0.5 * (h[a] + h[b])) / num[q];
            }
}

/* wrapper.F90:447-485: nothing when w is zero at every interior point */
void oracle_vertical_advection_to_sources(int nx_, int ny_, int nz, int halox, int haloy, const int *mask,
                                          const double *c, const double *w, const double *h, double *s)
{
    int active = 0;
    for (int k = 0; k < nz && !active; k++)
        for (int j = haloy; j < ny_ - haloy && !active; j++)
            for (int i = halox; i < nx_ - halox; i++)
                if (w[IDX3(i, j, k)] != 0.0) { active = 1; break; }
    if (!active) return;
    const double upward = -1.0;
    for (int k = 0; k < nz - 1; k++)
        for (int j = haloy; j < ny_ - haloy; j++)
            for (int i = halox; i < nx_ - halox; i++) {
                size_t a = IDX3(i, j, k), b = IDX3(i, j, k + 1);
                if (mask[a] == 1 && mask[b] == 1) {
                    double local_w = upward * 0.5 * (w[a] + w[b]);
                    double flux = local_w > 0.0 ? local_w * c[a] : local_w * c[b];
                    s[a] = s[a] - flux / h[a];
                    s[b] = s[b] + flux / h[b];
                }
            }
}

/* wrapper.F90:567-600 (kk 1-based) */
void oracle_update_gvc(int nx_, int ny_, int nz, double dsigma, const double *dbeta, double Dgamma, int kk,
                       const double *D, const int *mask, double *h)
{
    for (int j = 0; j < ny_; j++)
        for (int i = 0; i < nx_; i++) {
            size_t p = IDX2(i, j);
            double r = Dgamma / D[p];
            double alpha = ((r < 1.0 ? r : 1.0) * dsigma - dbeta[kk - 1]) / (dsigma - dbeta[kk - 1]);
            if (mask[p] == 0) continue;
            for (int k = 0; k < nz; k++) h[IDX3(i, j, k)] = D[p] * (dbeta[k] + alpha * (dsigma - dbeta[k]));
        }
}

/* momentum.F90:270-284 */
void oracle_surface_shear_velocity(int nx_, int ny_, int imin, int imax, int jmin, int jmax,
                                   const int *mask, const double *taux, const double *tauy,
                                   double *ustar)
{
    (void)ny_;
    const double rho0i = 1.0 / RHO0;
    for (int j = jmin - 1; j <= jmax - 1; j++)
        for (int i = imin - 1; i <= imax - 1; i++) {
            size_t p = IDX2(i, j);
            if (mask[p] > 0) ustar[p] = pow(taux[p] * taux[p] + tauy[p] * tauy[p], 0.25) * sqrt(rho0i);
        }
}

/* momentum.F90:286-321 */
void oracle_bottom_shear_velocity(int nx_, int ny_, int imin, int imax, int jmin, int jmax,
                                  const int *mask, const int *umask, const int *vmask,
                                  const double *uk_bot, const double *vk_bot, const double *rru,
                                  const double *rrv, double *ustar2_x, double *ustar2_y,
                                  double *ustar)
{
    (void)ny_; (void)umask; (void)vmask;
    for (int j = jmin - 1; j <= jmax - 1; j++)
        for (int i = 0; i < nx_; i++) {
            size_t p = IDX2(i, j);
            ustar2_x[p] = -uk_bot[p] * rru[p];
        }
    for (int j = jmin - 2; j <= jmax - 1; j++)
        for (int i = 0; i < nx_; i++) {
            size_t p = IDX2(i, j);
            ustar2_y[p] = -vk_bot[p] * rrv[p];
        }
    for (int j = jmin - 1; j <= jmax - 1; j++)
        for (int i = imin - 1; i <= imax - 1; i++) {
            size_t p = IDX2(i, j);
            if (mask[p] == 1) {
                double a = ustar2_x[p - 1], b = ustar2_x[p], c = ustar2_y[p - nx_], d = ustar2_y[p];
                ustar[p] = pow(0.5 * (a * a + b * b + c * c + d * d), 0.25);
            }
        }
}

/* momentum.F90:323-340 */
void oracle_reconstruct_transport_change(int nx_, int ny_, int nz, int imin, int imax, int jmin,
                                         int jmax, double *un, const double *hn, const double *Uo,
                                         double timestep)
{
    (void)imin; (void)imax;
    const double idt = 1.0 / timestep;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; k++)
        for (int j = jmin - 1; j <= jmax - 1; j++)
            for (int i = 0; i < nx_; i++) {
                size_t q = IDX3(i, j, k);
                un[q] = (un[q] * hn[q] - Uo[q]) * idt;
            }
}

/* ------------------------------------------------------------------------ */
/* python/src/internal_pressure.F90                                          */
/* ------------------------------------------------------------------------ */
/* internal_pressure.F90:9-60 */
void oracle_blumberg_mellor(int nx_, int ny_, int nz, int imin, int imax, int jmin, int jmax,
                            const int *umask, const int *vmask, const double *idxu,
                            const double *idyv, const double *hu, const double *hv,
                            const double *zf, const double *buoy, double *idpdx, double *idpdy)
{
    /* buoy/hu/idpdx level k (1..nz) -> plane k-1; zf level k (0..nz) -> plane k */
#define B(i, j, k) buoy[IDX3(i, j, (k) - 1)]
#pragma omp parallel for schedule(static)
    for (int j = jmin - 1; j <= jmax - 1; j++)
        for (int i = imin - 1; i <= imax - 1; i++) {
            size_t p = IDX2(i, j);
            if (umask[p] <= 0) continue;
            double grdl = (B(i + 1, j, nz) - B(i, j, nz)) * idxu[p];
            double buoyl = 0.5 * (B(i + 1, j, nz) + B(i, j, nz));
            double prgr = grdl * 0.5 * hu[IDX3(i, j, nz - 1)];
            idpdx[IDX3(i, j, nz - 1)] = hu[IDX3(i, j, nz - 1)] * prgr;
            for (int k = nz - 1; k >= 1; k--) {
                double grdu = grdl;
                grdl = (B(i + 1, j, k) - B(i, j, k)) * idxu[p];
                double buoyu = buoyl;
                buoyl = 0.5 * (B(i + 1, j, k) + B(i, j, k));
                double dxz = (zf[IDX3(i + 1, j, k)] - zf[IDX3(i, j, k)]) * idxu[p];
                prgr = prgr + 0.5 * (grdu + grdl) * 0.5 * (hu[IDX3(i, j, k - 1)] + hu[IDX3(i, j, k)]) - dxz * (buoyu - buoyl);
                idpdx[IDX3(i, j, k - 1)] = hu[IDX3(i, j, k - 1)] * prgr;
            }
        }
#pragma omp parallel for schedule(static)
    for (int j = jmin - 1; j <= jmax - 1; j++)
        for (int i = imin - 1; i <= imax - 1; i++) {
            size_t p = IDX2(i, j);
            if (vmask[p] <= 0) continue;
            double grdl = (B(i, j + 1, nz) - B(i, j, nz)) * idyv[p];
            double buoyl = 0.5 * (B(i, j + 1, nz) + B(i, j, nz));
            double prgr = grdl * 0.5 * hv[IDX3(i, j, nz - 1)];
            idpdy[IDX3(i, j, nz - 1)] = hv[IDX3(i, j, nz - 1)] * prgr;
            for (int k = nz - 1; k >= 1; k--) {
                double grdu = grdl;
                grdl = (B(i, j + 1, k) - B(i, j, k)) * idyv[p];
                double buoyu = buoyl;
                buoyl = 0.5 * (B(i, j + 1, k) + B(i, j, k));
                double dyz = (zf[IDX3(i, j + 1, k)] - zf[IDX3(i, j, k)]) * idyv[p];
                prgr = prgr + 0.5 * (grdu + grdl) * 0.5 * (hv[IDX3(i, j, k - 1)] + hv[IDX3(i, j, k)]) - dyz * (buoyu - buoyl);
                idpdy[IDX3(i, j, k - 1)] = hv[IDX3(i, j, k - 1)] * prgr;
            }
        }
#undef B
}

/* internal_pressure.F90:63-217 */
void oracle_shchepetkin_mcwilliams(int nx_, int ny_, int nz, int imin, int imax, int jmin, int jmax,
                                   const int *mask, const int *umask, const int *vmask,
                                   const double *idxu, const double *idyv, const double *h,
                                   const double *z, const double *zc, const double *buoy,
                                   double *idpdx, double *idpdy)
{
    const double eps = 1.e-10;
    const double x = 1.0 / 12.0;
    const size_t n2 = (size_t)nx_ * ny_;
    /* dR, dZ have levels 0..nz (plane k); P levels 1..nz (plane k-1) */
    double *dR = (double *)calloc(n2 * (nz + 1), sizeof(double));
    double *dZ = (double *)calloc(n2 * (nz + 1), sizeof(double));
    double *P = (double *)calloc(n2 * nz, sizeof(double));
    double *dZx = (double *)calloc(n2, sizeof(double));
    double *dRx = (double *)calloc(n2, sizeof(double));
#define B(i, j, k) buoy[IDX3(i, j, (k) - 1)]
#define ZC(i, j, k) zc[IDX3(i, j, (k) - 1)]
#define HH(i, j, k) h[IDX3(i, j, (k) - 1)]
#define DR(i, j, k) dR[IDX3(i, j, k)]
#define DZ(i, j, k) dZ[IDX3(i, j, k)]
#define PP(i, j, k) P[IDX3(i, j, (k) - 1)]
    /* :80-118  (C i in imin-1..imax, j in jmin-1..jmax: Fortran imin..imax+1) */
#pragma omp parallel for schedule(static)
    for (int j = jmin - 1; j <= jmax; j++)
        for (int i = imin - 1; i <= imax; i++) {
            if (mask[IDX2(i, j)] <= 0) continue;
            for (int k = nz - 1; k >= 1; k--) {
                DR(i, j, k) = B(i, j, k + 1) - B(i, j, k);
                DZ(i, j, k) = ZC(i, j, k + 1) - ZC(i, j, k);
            }
            DR(i, j, nz) = DR(i, j, nz - 1);
            DZ(i, j, nz) = DZ(i, j, nz - 1);
            DR(i, j, 0) = DR(i, j, 1);
            DZ(i, j, 0) = DZ(i, j, 1);
            for (int k = nz; k >= 1; k--) {
                double cff = 2.0 * DR(i, j, k) * DR(i, j, k - 1);
                if (cff > eps)
                    DR(i, j, k) = cff / (DR(i, j, k) + DR(i, j, k - 1));
                else
                    DR(i, j, k) = 0.0;
                DZ(i, j, k) = 2.0 * DZ(i, j, k) * DZ(i, j, k - 1) / (DZ(i, j, k) + DZ(i, j, k - 1));
            }
            double cff;
            if (nz > 1)
                cff = 0.5 * (B(i, j, nz) - B(i, j, nz - 1)) * 0.5 * HH(i, j, nz) / (ZC(i, j, nz) - ZC(i, j, nz - 1));
            else
                cff = 0.0;
            PP(i, j, nz) = (B(i, j, nz) + cff) * 0.5 * HH(i, j, nz);
            for (int k = nz - 1; k >= 1; k--)
                PP(i, j, k) = PP(i, j, k + 1) + 0.5 * ((B(i, j, k + 1) + B(i, j, k)) * (ZC(i, j, k + 1) - ZC(i, j, k))
                    - 0.2 * ((DR(i, j, k + 1) - DR(i, j, k)) * (ZC(i, j, k + 1) - ZC(i, j, k) - x * (DZ(i, j, k + 1) + DZ(i, j, k)))
                    - (DZ(i, j, k + 1) - DZ(i, j, k)) * (B(i, j, k + 1) - B(i, j, k) - x * (DR(i, j, k + 1) + DR(i, j, k)))));
        }
    /* x-direction :120-167 */
    for (int k = nz; k >= 1; k--) {
#pragma omp parallel for schedule(static)
        for (int j = jmin - 1; j <= jmax - 1; j++)
            for (int i = imin - 1; i <= imax + 1; i++) {
                size_t p = IDX2(i, j);
                if (umask[p - 1] > 0) {
                    dZx[p] = ZC(i, j, k) - ZC(i - 1, j, k);
                    dRx[p] = B(i, j, k) - B(i - 1, j, k);
                } else {
                    dZx[p] = 0.0;
                    dRx[p] = 0.0;
                }
            }
#pragma omp parallel for schedule(static)
        for (int j = jmin - 1; j <= jmax - 1; j++)
            for (int i = imin - 1; i <= imax; i++) {
                size_t p = IDX2(i, j);
                double cff = 2.0 * dZx[p] * dZx[p + 1];
                dZx[p] = (cff > eps) ? cff / (dZx[p] + dZx[p + 1]) : 0.0;
                cff = 2.0 * dRx[p] * dRx[p + 1];
                dRx[p] = (cff > eps) ? cff / (dRx[p] + dRx[p + 1]) : 0.0;
            }
#pragma omp parallel for schedule(static)
        for (int j = jmin - 1; j <= jmax - 1; j++)
            for (int i = imin - 1; i <= imax - 1; i++) {
                size_t p = IDX2(i, j);
                if (umask[p] != 1) continue;
                double FC = 0.5 * ((B(i + 1, j, k) + B(i, j, k)) * (ZC(i + 1, j, k) - ZC(i, j, k))
                    - 0.2 * ((dRx[p + 1] - dRx[p]) * (ZC(i + 1, j, k) - ZC(i, j, k) - x * (dZx[p + 1] + dZx[p]))
                    - (dZx[p + 1] - dZx[p]) * (B(i + 1, j, k) - B(i, j, k) - x * (dRx[p + 1] + dRx[p]))));
                idpdx[IDX3(i, j, k - 1)] = 0.5 * (HH(i, j, k) + HH(i + 1, j, k)) * idxu[p]
                    * (PP(i + 1, j, k) - PP(i, j, k) + FC - (z[p + 1] - z[p]) * 0.5 * (B(i + 1, j, nz) + B(i, j, nz)));
            }
    }
    /* y-direction :169-216 */
    for (int k = nz; k >= 1; k--) {
#pragma omp parallel for schedule(static)
        for (int j = jmin - 1; j <= jmax + 1; j++)
            for (int i = imin - 1; i <= imax - 1; i++) {
                size_t p = IDX2(i, j);
                if (vmask[p - nx_] > 0) {
                    dZx[p] = ZC(i, j, k) - ZC(i, j - 1, k);
                    dRx[p] = B(i, j, k) - B(i, j - 1, k);
                } else {
                    dZx[p] = 0.0;
                    dRx[p] = 0.0;
                }
            }
#pragma omp parallel for schedule(static)
        for (int j = jmin - 1; j <= jmax; j++)
            for (int i = imin - 1; i <= imax - 1; i++) {
                size_t p = IDX2(i, j);
                double cff = 2.0 * dZx[p] * dZx[p + nx_];
                dZx[p] = (cff > eps) ? cff / (dZx[p] + dZx[p + nx_]) : 0.0;
                cff = 2.0 * dRx[p] * dRx[p + nx_];
                dRx[p] = (cff > eps) ? cff / (dRx[p] + dRx[p + nx_]) : 0.0;
            }
#pragma omp parallel for schedule(static)
        for (int j = jmin - 1; j <= jmax - 1; j++)
            for (int i = imin - 1; i <= imax - 1; i++) {
                size_t p = IDX2(i, j);
                if (vmask[p] != 1) continue;
                double FC = 0.5 * ((B(i, j + 1, k) + B(i, j, k)) * (ZC(i, j + 1, k) - ZC(i, j, k))
                    - 0.2 * ((dRx[p + nx_] - dRx[p]) * (ZC(i, j + 1, k) - ZC(i, j, k) - x * (dZx[p + nx_] + dZx[p]))
                    - (dZx[p + nx_] - dZx[p]) * (B(i, j + 1, k) - B(i, j, k) - x * (dRx[p + nx_] + dRx[p]))));
                idpdy[IDX3(i, j, k - 1)] = 0.5 * (HH(i, j, k) + HH(i, j + 1, k)) * idyv[p]
                    * (PP(i, j + 1, k) - PP(i, j, k) + FC - (z[p + nx_] - z[p]) * 0.5 * (B(i, j + 1, nz) + B(i, j, nz)));
            }
    }
#undef B
#undef ZC
#undef HH
#undef DR
#undef DZ
#undef PP
    free(dR); free(dZ); free(P); free(dZx); free(dRx);
}
