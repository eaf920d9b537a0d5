// Grid utilities of python/src/wrapper.F90 and python/src/interpolation.F90
// for sm_103a: staggered interpolation, depth/thickness bookkeeping, the
// surface-elevation update and the surface pressure gradient.
//
// These are elementwise or single-pass column kernels; each thread owns one
// output point (or one column for the vertical recursions), reads its inputs
// once, and warps run along i so every access is coalesced.
#include "split2d_ops.cuh"

#define EW_THREADS 256

#include <atomic>

static std::atomic<unsigned long long> g_launches{0};

extern "C" unsigned long long getm_launch_counter_add(void) { return ++g_launches; }

extern "C" int getm_launch_count(unsigned long long* count)
{
    if (!count) return GETM_ERR_ARG;
    *count = g_launches.load();
    return GETM_OK;
}

// ---------------------------------------------------------------------------
// interpolation.F90:9-72 (T: double for the FP64 form, float for the mixed form)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void interp_x_kernel(int nx, int ny, int nz, const T* s, T* t, int ioff)
{
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n = (long long)nx * ny * nz;
    if (p >= n) return;
    int i = (int)(p % nx);
    if (i >= nx - 1) return;
    interp_pair_point<T>(s, t, p, 1, ioff);
}

template <typename T>
__global__ void interp_y_kernel(int nx, int ny, int nz, const T* s, T* t, int joff)
{
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n = (long long)nx * ny * nz;
    if (p >= n) return;
    int j = (int)((p / nx) % ny);
    if (j >= ny - 1) return;
    interp_pair_point<T>(s, t, p, nx, (long long)joff * nx);
}

template <typename T>
__global__ void interp_z_kernel(int nx, int ny, int nz1, const T* s, T* t, int koff)
{
    long long plane = (long long)nx * ny;
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= plane * (nz1 - 1)) return;
    t[p + koff * plane] = T(0.5) * (s[p] + s[p + plane]);
}

template <typename T>
__global__ void interp_xy_kernel(int nx1, int ny1, int nx2, int ny2, int nz, const T* s, T* t, int ioff, int joff)
{
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n = (long long)(nx1 - 1) * (ny1 - 1) * nz;
    if (p >= n) return;
    int i = (int)(p % (nx1 - 1));
    long long r = p / (nx1 - 1);
    int j = (int)(r % (ny1 - 1));
    int k = (int)(r / (ny1 - 1));
    long long q = ((long long)k * ny1 + j) * nx1 + i;
    t[((long long)k * ny2 + j + joff) * nx2 + i + ioff] = T(0.25) * (s[q] + s[q + 1] + s[q + nx1] + s[q + nx1 + 1]);
}

template <typename T>
static int interp_x_impl(int nx, int ny, int nz, const T* source, T* target, int ioffset, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || !source || !target) return GETM_ERR_ARG;
    long long n = (long long)nx * ny * nz;
    interp_x_kernel<T><<<getm_div_up(n, EW_THREADS), EW_THREADS, 0, stream>>>(nx, ny, nz, source, target, ioffset);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

template <typename T>
static int interp_y_impl(int nx, int ny, int nz, const T* source, T* target, int joffset, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || !source || !target) return GETM_ERR_ARG;
    long long n = (long long)nx * ny * nz;
    interp_y_kernel<T><<<getm_div_up(n, EW_THREADS), EW_THREADS, 0, stream>>>(nx, ny, nz, source, target, joffset);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

template <typename T>
static int interp_z_impl(int nx, int ny, int nz1, int nz2, const T* source, T* target, int koffset,
                         cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz1 < 1 || nz2 < 1 || !source || !target) return GETM_ERR_ARG;
    if (nz1 < 2) return GETM_OK;
    long long n = (long long)nx * ny * (nz1 - 1);
    interp_z_kernel<T><<<getm_div_up(n, EW_THREADS), EW_THREADS, 0, stream>>>(nx, ny, nz1, source, target, koffset);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

template <typename T>
static int interp_xy_impl(int nx1, int ny1, int nx2, int ny2, int nz, const T* source, T* target, int ioffset,
                          int joffset, cudaStream_t stream)
{
    if (nx1 < 1 || ny1 < 1 || nx2 < 1 || ny2 < 1 || nz < 1 || !source || !target) return GETM_ERR_ARG;
    if (nx1 < 2 || ny1 < 2) return GETM_OK;
    long long n = (long long)(nx1 - 1) * (ny1 - 1) * nz;
    interp_xy_kernel<T><<<getm_div_up(n, EW_THREADS), EW_THREADS, 0, stream>>>(nx1, ny1, nx2, ny2, nz, source, target, ioffset, joffset);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_grid_interp_x(int nx, int ny, int nz, const double* source, double* target, int ioffset,
                                  cudaStream_t stream)
{
    return interp_x_impl<double>(nx, ny, nz, source, target, ioffset, stream);
}

extern "C" int getm_grid_interp_y(int nx, int ny, int nz, const double* source, double* target, int joffset,
                                  cudaStream_t stream)
{
    return interp_y_impl<double>(nx, ny, nz, source, target, joffset, stream);
}

extern "C" int getm_grid_interp_z(int nx, int ny, int nz1, int nz2, const double* source, double* target,
                                  int koffset, cudaStream_t stream)
{
    return interp_z_impl<double>(nx, ny, nz1, nz2, source, target, koffset, stream);
}

extern "C" int getm_grid_interp_xy(int nx1, int ny1, int nx2, int ny2, int nz, const double* source, double* target,
                                   int ioffset, int joffset, cudaStream_t stream)
{
    return interp_xy_impl<double>(nx1, ny1, nx2, ny2, nz, source, target, ioffset, joffset, stream);
}

extern "C" int getm_grid_interp_x_f32(int nx, int ny, int nz, const float* source, float* target, int ioffset,
                                      cudaStream_t stream)
{
    return interp_x_impl<float>(nx, ny, nz, source, target, ioffset, stream);
}

extern "C" int getm_grid_interp_y_f32(int nx, int ny, int nz, const float* source, float* target, int joffset,
                                      cudaStream_t stream)
{
    return interp_y_impl<float>(nx, ny, nz, source, target, joffset, stream);
}

extern "C" int getm_grid_interp_z_f32(int nx, int ny, int nz1, int nz2, const float* source, float* target,
                                      int koffset, cudaStream_t stream)
{
    return interp_z_impl<float>(nx, ny, nz1, nz2, source, target, koffset, stream);
}

extern "C" int getm_grid_interp_xy_f32(int nx1, int ny1, int nx2, int ny2, int nz, const float* source,
                                       float* target, int ioffset, int joffset, cudaStream_t stream)
{
    return interp_xy_impl<float>(nx1, ny1, nx2, ny2, nz, source, target, ioffset, joffset, stream);
}

// ---------------------------------------------------------------------------
// wrapper.F90 utilities
// ---------------------------------------------------------------------------
__global__ void elevation2depth_kernel(int n, const double* z, const double* H, double Dmin,
                                       const int* mask, double* D)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n && mask[p] != 0) D[p] = fmax(H[p] + z[p], Dmin);  // wrapper.F90:444
}

// wrapper.F90:428-436, with the constant divisor 1/(Dcrit - Dmin) formed once
// (ialpha) and applied as a product: FP64 division is costly on GB300.
__global__ void alpha_kernel(int n, const double* D, double Dmin, double ialpha, const int* mask,
                             double* alpha)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n && mask[p] != 0)  // wrapper.F90:434
        alpha[p] = fmax(0.0, fmin(1.0, (D[p] - Dmin) * ialpha));
}

__global__ void multiply_add_kernel(int n, double* tgt, const double* add, double s)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) tgt[p] = tgt[p] + s * add[p];  // wrapper.F90:493
}

extern "C" int getm_elevation2depth(int n, const double* z, const double* H, double Dmin,
                                    const int* mask, double* D, cudaStream_t stream)
{
    if (n < 0 || !z || !H || !mask || !D) return GETM_ERR_ARG;
    if (n == 0) return GETM_OK;
    elevation2depth_kernel<<<getm_div_up(n, EW_THREADS), EW_THREADS, 0, stream>>>(n, z, H, Dmin, mask, D);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_alpha(int n, const double* D, double Dmin, double Dcrit, const int* mask,
                          double* alpha, cudaStream_t stream)
{
    if (n < 0 || !D || !mask || !alpha) return GETM_ERR_ARG;
    if (n == 0) return GETM_OK;
    alpha_kernel<<<getm_div_up(n, EW_THREADS), EW_THREADS, 0, stream>>>(n, D, Dmin, 1.0 / (Dcrit - Dmin), mask, alpha);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_multiply_add(int n, double* tgt, const double* add, double scale_factor,
                                 cudaStream_t stream)
{
    if (n < 0 || (n > 0 && (!tgt || !add))) return GETM_ERR_ARG;
    if (n == 0) return GETM_OK;
    multiply_add_kernel<<<getm_div_up(n, EW_THREADS), EW_THREADS, 0, stream>>>(n, tgt, add, scale_factor);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// wrapper.F90:409-426: column recursion, thread per column
// thickness2vertical_coordinates of the column at p (wrapper.F90:409-426)
__device__ __forceinline__ void t2vc_column(long long plane, int nz, long long p, const double* __restrict__ bd,
                                            const double* __restrict__ h, double* __restrict__ zc,
                                            double* __restrict__ zf)
{
    double zci = -bd[p] + 0.5 * h[p];
    zc[p] = zci;
    double hprev = h[p];
    for (int k = 1; k < nz; k++) {
        double hk = h[p + k * plane];
        zci = zci + 0.5 * (hprev + hk);
        zc[p + k * plane] = zci;
        hprev = hk;
    }
    double zfi = -bd[p];
    zf[p] = zfi;
    for (int k = 1; k <= nz; k++) {
        zfi = zfi + h[p + (k - 1) * plane];
        zf[p + k * plane] = zfi;
    }
}

__global__ void t2vc_kernel(int nx, int ny, int nz, const int* mask, const double* bd,
                            const double* h, double* zc, double* zf)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    long long plane = (long long)nx * ny;
    if (p >= plane || mask[p] == 0) return;
    t2vc_column(plane, nz, p, bd, h, zc, zf);
}

extern "C" int getm_thickness2vertical_coordinates(int nx, int ny, int nz, const int* mask,
                                                   const double* bottom_depth, const double* h,
                                                   double* zc, double* zf, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || !mask || !bottom_depth || !h || !zc || !zf) return GETM_ERR_ARG;
    int n = nx * ny;
    t2vc_kernel<<<getm_div_up(n, 128), 128, 0, stream>>>(nx, ny, nz, mask, bottom_depth, h, zc, zf);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// wrapper.F90:395-407: depth of the layer centres below the surface
__device__ __forceinline__ void t2cd_column(long long plane, int nz, long long p, const double* __restrict__ h,
                                            double* __restrict__ out)
{
    double hk1 = h[p + (nz - 1) * plane];
    double o = 0.5 * hk1;
    out[p + (nz - 1) * plane] = o;
    for (int k = nz - 2; k >= 0; k--) {
        double hk = h[p + k * plane];
        o = o + 0.5 * (hk + hk1);
        out[p + k * plane] = o;
        hk1 = hk;
    }
}

__global__ void t2cd_kernel(int nx, int ny, int nz, const int* mask, const double* h, double* out)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    long long plane = (long long)nx * ny;
    if (p >= plane || mask[p] == 0) return;
    t2cd_column(plane, nz, p, h, out);
}

extern "C" int getm_thickness2center_depth(int nx, int ny, int nz, int istart, int istop, int jstart,
                                           int jstop, const int* mask, const double* h, double* out,
                                           cudaStream_t stream)
{
    (void)istart; (void)istop; (void)jstart; (void)jstop;  // unused by the reference too
    if (nx < 1 || ny < 1 || nz < 1 || !mask || !h || !out) return GETM_ERR_ARG;
    int n = nx * ny;
    t2cd_kernel<<<getm_div_up(n, 128), 128, 0, stream>>>(nx, ny, nz, mask, h, out);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// wrapper.F90:496-523
__global__ void surface_elevation_kernel(int nx, int ny, int halox, int haloy, const int* mask,
                                         const double* dyu, const double* dxv,
                                         const double* iarea, double* z, const double* U,
                                         const double* V, const double* fwf, double dt)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i < halox || i >= nx - halox || j < haloy || j >= ny - haloy) return;
    long long p = (long long)j * nx + i;
    if (mask[p] != 1) return;
    z[p] = z[p] + dt * ((U[p - 1] * dyu[p - 1] - U[p] * dyu[p] + V[p - nx] * dxv[p - nx] - V[p] * dxv[p]) * iarea[p] + fwf[p]);
}

extern "C" int getm_advance_surface_elevation(int nx, int ny, int halox, int haloy, const int* mask,
                                              const double* dyu, const double* dxv,
                                              const double* iarea, double* z, const double* U,
                                              const double* V, const double* fwf, double dt,
                                              cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || halox < 1 || haloy < 1 || !mask || !dyu || !dxv || !iarea || !z || !U || !V || !fwf)
        return GETM_ERR_ARG;
    dim3 grid(getm_div_up(nx, 128), ny);
    surface_elevation_kernel<<<grid, 128, 0, stream>>>(nx, ny, halox, haloy, mask, dyu, dxv, iarea, z, U, V, fwf, dt);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// wrapper.F90:525-565; C bounds from Fortran 1-based imin..jmax
__global__ void spg_kernel(int nx, int ny, int ilo, int ihi, int jlo, int jhi, SpgArgs a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i < ilo || i > ihi || j < jlo || j > jhi) return;
    spg_point(a, (long long)j * nx + i);
}

extern "C" int getm_surface_pressure_gradient(int nx, int ny, int imin, int imax, int jmin, int jmax,
                                              const int* umask, const int* vmask, const double* idxu,
                                              const double* idyv, const double* z, const double* sp,
                                              const double* H, const double* D, double Dmin,
                                              double* dpdx, double* dpdy, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || imin < 1 || jmin < 1 || imax >= nx || jmax >= ny) return GETM_ERR_ARG;
    if (!umask || !vmask || !idxu || !idyv || !z || !sp || !H || !D || !dpdx || !dpdy) return GETM_ERR_ARG;
    dim3 grid(getm_div_up(nx, 128), ny);
    SpgArgs a{nx, umask, vmask, idxu, idyv, z, sp, H, D, Dmin, dpdx, dpdy};
    spg_kernel<<<grid, 128, 0, stream>>>(nx, ny, imin - 1, imax - 1, jmin - 1, jmax - 1, a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// ---------------------------------------------------------------------------
// Simulation.update_depth, 3D part (python/pygetm/simulation.py:1588-1630) in
// three launches.  1 (one thread per point and level of every grid): ho = hn;
// hn = dga Dclip where the mask is non-zero (Sigma coordinates,
// vertical_coordinates.py:106-113).  2 (per point and level, needs the new
// thicknesses of neighbouring columns): h_T_half = (ho + hn) / 2 on T and the
// thicknesses of the advection velocity grids (UU from h_T_half at i+1, VV
// at j+1, UV = VU = X at (j+1, i+1)).  3 (per column): the vertical
// coordinates of T, U, V and the T centre depths.  Same arithmetic as the
// separate array operations.
// ---------------------------------------------------------------------------
struct Depth3DArgs {
    int nx, ny, nz;
    long long plane, planex;
    const double* dga;
    const int *mt, *mu, *mv, *mx;
    const double *Dt, *Du, *Dv, *Dx;      // Dclip of each grid
    const double *Ht, *Hu, *Hv;
    double *hnt, *hnu, *hnv, *hnx;
    double *hot, *hou, *hov;
    double *zct, *zcu, *zcv, *zft, *zfu, *zfv;
    double* depth;                         // T centre depths, or NULL
    double *hhalf, *hnuu, *hnvv, *hnuv, *hnvu;
};

__device__ __forceinline__ void sigma_point(double dga, long long p, long long q, const int* __restrict__ m,
                                            const double* __restrict__ D, double* __restrict__ hn,
                                            double* __restrict__ ho)
{
    const double old = hn[q];
    if (ho) ho[q] = old;
    hn[q] = m[p] != 0 ? dga * D[p] : old;
}

// grid (ceil((nx + 1) / 128), ny + 1, nz)
__global__ void depth_3d_sigma_kernel(Depth3DArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    const double dga = a.dga[k];
    if (i <= a.nx && j <= a.ny) {  // X grid: (ny + 1) x (nx + 1)
        const long long px = (long long)j * (a.nx + 1) + i;
        sigma_point(dga, px, px + k * a.planex, a.mx, a.Dx, a.hnx, nullptr);
    }
    if (i >= a.nx || j >= a.ny) return;
    const long long p = (long long)j * a.nx + i, q = p + k * a.plane;
    sigma_point(dga, p, q, a.mt, a.Dt, a.hnt, a.hot);
    sigma_point(dga, p, q, a.mu, a.Du, a.hnu, a.hou);
    sigma_point(dga, p, q, a.mv, a.Dv, a.hnv, a.hov);
}

// grid (ceil(nx / 128), ny, nz)
__global__ void depth_3d_halves_kernel(Depth3DArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= a.nx || j >= a.ny) return;
    const long long p = (long long)j * a.nx + i, q = p + k * a.plane;
    const double hh = (a.hot[q] + a.hnt[q]) * 0.5;
    a.hhalf[q] = hh;
    if (i >= 1) a.hnuu[q - 1] = hh;     // UU.hn[:, :, :-1] = h_T_half[:, :, 1:]
    if (j >= 1) a.hnvv[q - a.nx] = hh;  // VV.hn[:, :-1, :] = h_T_half[:, 1:, :]
    const double hx = a.hnx[(long long)(j + 1) * (a.nx + 1) + (i + 1) + k * a.planex];
    a.hnuv[q] = hx;                     // UV.hn = X.hn[:, 1:, 1:]
    a.hnvu[q] = hx;                     // VU.hn = UV.hn
}

// one thread per column
__global__ void depth_3d_coords_kernel(Depth3DArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= a.nx || j >= a.ny) return;
    const long long p = (long long)j * a.nx + i;
    if (a.mt[p] != 0) {
        t2vc_column(a.plane, a.nz, p, a.Ht, a.hnt, a.zct, a.zft);
        if (a.depth) t2cd_column(a.plane, a.nz, p, a.hnt, a.depth);
    }
    if (a.mu[p] != 0) t2vc_column(a.plane, a.nz, p, a.Hu, a.hnu, a.zcu, a.zfu);
    if (a.mv[p] != 0) t2vc_column(a.plane, a.nz, p, a.Hv, a.hnv, a.zcv, a.zfv);
}

extern "C" int getm_update_depth_3d(const getm_depth3d_fields* f, int nx, int ny, int nz, cudaStream_t stream)
{
    if (!f || nx < 2 || ny < 2 || nz < 1) return GETM_ERR_ARG;
    const void* ptrs[] = {f->dga, f->mask_t, f->mask_u, f->mask_v, f->mask_x, f->Dclip_t, f->Dclip_u, f->Dclip_v,
                          f->Dclip_x, f->H_t, f->H_u, f->H_v, f->hn_t, f->hn_u, f->hn_v, f->hn_x, f->ho_t, f->ho_u,
                          f->ho_v, f->zc_t, f->zc_u, f->zc_v, f->zf_t, f->zf_u, f->zf_v, f->h_T_half, f->hn_uu,
                          f->hn_vv, f->hn_uv, f->hn_vu};
    for (const void* q : ptrs)
        if (!q) return GETM_ERR_ARG;
    Depth3DArgs a{nx, ny, nz, (long long)nx * ny, (long long)(nx + 1) * (ny + 1), f->dga,
                  f->mask_t, f->mask_u, f->mask_v, f->mask_x, f->Dclip_t, f->Dclip_u, f->Dclip_v, f->Dclip_x,
                  f->H_t, f->H_u, f->H_v, f->hn_t, f->hn_u, f->hn_v, f->hn_x, f->ho_t, f->ho_u, f->ho_v,
                  f->zc_t, f->zc_u, f->zc_v, f->zf_t, f->zf_u, f->zf_v, f->depth,
                  f->h_T_half, f->hn_uu, f->hn_vv, f->hn_uv, f->hn_vu};
    depth_3d_sigma_kernel<<<dim3(getm_div_up(nx + 1, 128), ny + 1, nz), 128, 0, stream>>>(a);
    GETM_CHECK_LAUNCH();
    depth_3d_halves_kernel<<<dim3(getm_div_up(nx, 128), ny, nz), 128, 0, stream>>>(a);
    GETM_CHECK_LAUNCH();
    depth_3d_coords_kernel<<<dim3(getm_div_up(nx, 128), ny), 128, 0, stream>>>(a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}
