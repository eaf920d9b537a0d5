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

__global__ void advance_time_kernel(double* time, double dt) { *time = *time + dt; }

extern "C" int getm_advance_time(double* time, double timestep, cudaStream_t stream)
{
    if (!time) return GETM_ERR_ARG;
    advance_time_kernel<<<1, 1, 0, stream>>>(time, timestep);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_stream_create(int priority, cudaStream_t* stream)
{
    if (!stream) return GETM_ERR_ARG;
    return cudaStreamCreateWithPriority(stream, cudaStreamNonBlocking, priority) == cudaSuccess ? GETM_OK
                                                                                              : GETM_ERR_CUDA;
}

extern "C" int getm_stream_destroy(cudaStream_t stream)
{
    return cudaStreamDestroy(stream) == cudaSuccess ? GETM_OK : GETM_ERR_CUDA;
}

extern "C" int getm_graph_launch(void* graph_exec, cudaStream_t stream)
{
    if (!graph_exec) return GETM_ERR_ARG;
    return cudaGraphLaunch((cudaGraphExec_t)graph_exec, stream) == cudaSuccess ? GETM_OK : GETM_ERR_CUDA;
}

// Launch-shape knobs, per host thread (a thread that captures a domain's
// graphs sets its own shapes without disturbing another thread's launches).
static thread_local int g_tune[GETM_TUNE_NKNOBS] = {8, 32, 4, 0, 1, 0};

static bool tune_valid(int knob, int v)
{
    switch (knob) {
    case GETM_TUNE_XPASS_ROWS: return v == 2 || v == 4 || v == 8;
    case GETM_TUNE_YMARCH_CHUNK: return v == 16 || v == 32 || v == 64;
    case GETM_TUNE_COLUMN_ROWS: return v == 1 || v == 2 || v == 4;
    case GETM_TUNE_SUBSTEP_BLOCKS: return v >= 0 && v <= 2;
    case GETM_TUNE_XPASS_VEC: return v == 0 || v == 1;
    case GETM_TUNE_COLUMN_SOLVE: return v == 0 || v == 1;
    default: return false;
    }
}

int getm_tune(int knob) { return (knob >= 0 && knob < GETM_TUNE_NKNOBS) ? g_tune[knob] : 0; }

extern "C" int getm_tune_set(int knob, int value)
{
    if (!tune_valid(knob, value)) return GETM_ERR_ARG;
    g_tune[knob] = value;
    return GETM_OK;
}

extern "C" int getm_tune_get(int knob, int* value)
{
    if (!value || knob < 0 || knob >= GETM_TUNE_NKNOBS) return GETM_ERR_ARG;
    *value = g_tune[knob];
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
template <bool MIXED>
__global__ void spg_kernel(int nx, int ny, int ilo, int ihi, int jlo, int jhi, SpgArgs a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i < ilo || i > ihi || j < jlo || j > jhi) return;
    spg_point<MIXED>(a, (long long)j * nx + i);
}

template <bool MIXED>
static int spg_impl(int nx, int ny, int imin, int imax, int jmin, int jmax, const int* umask, const int* vmask,
                    const double* idxu, const double* idyv, const double* z, const double* sp, const double* H,
                    const double* D, double Dmin, double* dpdx, double* dpdy, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || imin < 1 || jmin < 1 || imax >= nx || jmax >= ny) return GETM_ERR_ARG;
    if (!umask || !vmask || !idxu || !idyv || !z || !sp || !H || !D || !dpdx || !dpdy) return GETM_ERR_ARG;
    dim3 grid(getm_div_up(nx, 128), ny);
    SpgArgs a{nx, umask, vmask, idxu, idyv, z, sp, H, D, Dmin, dpdx, dpdy};
    spg_kernel<MIXED><<<grid, 128, 0, stream>>>(nx, ny, imin - 1, imax - 1, jmin - 1, jmax - 1, a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_surface_pressure_gradient(int nx, int ny, int imin, int imax, int jmin, int jmax,
                                              const int* umask, const int* vmask, const double* idxu,
                                              const double* idyv, const double* z, const double* sp,
                                              const double* H, const double* D, double Dmin,
                                              double* dpdx, double* dpdy, cudaStream_t stream)
{
    return spg_impl<false>(nx, ny, imin, imax, jmin, jmax, umask, vmask, idxu, idyv, z, sp, H, D, Dmin, dpdx, dpdy,
                           stream);
}

extern "C" int getm_surface_pressure_gradient_mixed(int nx, int ny, int imin, int imax, int jmin, int jmax,
                                                    const int* umask, const int* vmask, const double* idxu,
                                                    const double* idyv, const double* z, const double* sp,
                                                    const double* H, const double* D, double Dmin,
                                                    double* dpdx, double* dpdy, cudaStream_t stream)
{
    return spg_impl<true>(nx, ny, imin, imax, jmin, jmax, umask, vmask, idxu, idyv, z, sp, H, D, Dmin, dpdx, dpdy,
                          stream);
}

// ---------------------------------------------------------------------------
// Simulation.update_depth, 3D part (python/pygetm/simulation.py:1588-1630) in
// one launch, one thread per column of each grid (X: 0 <= j <= ny,
// 0 <= i <= nx; T, U, V: j < ny, i < nx), sweeping up from the bottom:
// hn = dga Dclip where the mask is non-zero
// (Sigma coordinates, vertical_coordinates.py:106-113) on X and, for j < ny
// and i < nx, on T, U and V with ho = the previous hn; h_T_half = (ho + hn) / 2
// on T and the thicknesses of the advection velocity grids, each written by
// the thread that owns its source value (UU.hn(j, i-1) = VV.hn(j-1, i) =
// h_T_half(j, i), UV.hn(j-1, i-1) = VU.hn(j-1, i-1) = X.hn(j, i)); the
// vertical coordinates of T, U and V accumulate in the same sweep and the T
// centre depths follow in a second, downward sweep over the new T
// thicknesses.  Same arithmetic as the separate array operations.
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

// one level of the upward coordinate sweep of a column (t2vc_column's
// arithmetic): zc(k) from zc(k-1) and the mean of the two thicknesses, zf(k+1)
// = zf(k) + h(k)
struct CoordSweep {
    double zc, zf, hprev;
    __device__ __forceinline__ void level(int k, long long q, long long plane, double H, double hk, double* zcp,
                                          double* zfp)
    {
        if (k == 0) {
            zc = -H + 0.5 * hk;
            zf = -H;
            zfp[q] = zf;
        } else {
            zc = zc + 0.5 * (hprev + hk);
        }
        zcp[q] = zc;
        zf = zf + hk;
        zfp[q + plane] = zf;
        hprev = hk;
    }
};

// One role per blockIdx.y, flattened over the (nx + 1) x (ny + 1) X-grid
// columns: 0 the X grid (and the UV/VU thicknesses it feeds), 1 T (with
// h_T_half, the UU/VV thicknesses and the centre depths), 2 U, 3 V.  The roles
// share no intermediate value, so splitting them keeps few values live per
// thread and four times the columns in flight.
__global__ void depth_3d_column_kernel(Depth3DArgs a)
{
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int role = blockIdx.y;
    int i, j;
    if (!getm_flat_column(nx + 1, 0, ny + 1, i, j)) return;
    const long long plane = a.plane;
    if (role == 0) {
        const long long px = (long long)j * (nx + 1) + i;
        const bool xm = a.mx[px] != 0;
        const double Dx = xm ? a.Dx[px] : 0.0;
        const bool xuv = i >= 1 && j >= 1;
        const long long quv = (long long)(j - 1) * nx + (i - 1);
        for (int k = 0; k < nz; k++) {
            const long long qx = px + k * a.planex;
            double hx;
            if (xm) {
                hx = a.dga[k] * Dx;
                a.hnx[qx] = hx;
            } else {
                hx = a.hnx[qx];
            }
            if (xuv) {
                a.hnuv[quv + k * plane] = hx;
                a.hnvu[quv + k * plane] = hx;
            }
        }
        return;
    }
    if (i >= nx || j >= ny) return;
    const long long p = (long long)j * nx + i;
    const int* mask = role == 1 ? a.mt : role == 2 ? a.mu : a.mv;
    const double* Dc = role == 1 ? a.Dt : role == 2 ? a.Du : a.Dv;
    const double* Hc = role == 1 ? a.Ht : role == 2 ? a.Hu : a.Hv;
    double* hn = role == 1 ? a.hnt : role == 2 ? a.hnu : a.hnv;
    double* ho = role == 1 ? a.hot : role == 2 ? a.hou : a.hov;
    double* zc = role == 1 ? a.zct : role == 2 ? a.zcu : a.zcv;
    double* zf = role == 1 ? a.zft : role == 2 ? a.zfu : a.zfv;
    const bool m = mask[p] != 0;
    const double D = m ? Dc[p] : 0.0, H = m ? Hc[p] : 0.0;
    CoordSweep sw{0.0, 0.0, 0.0};
    // the old thicknesses of DEPTH3D_CHUNK levels are loaded before any of
    // their stores (the stores may alias as far as the compiler knows, which
    // would serialise each level's load behind the previous level's stores)
    constexpr int DEPTH3D_CHUNK = 8;
    for (int k0 = 0; k0 < nz; k0 += DEPTH3D_CHUNK) {
        double ov[DEPTH3D_CHUNK];
#pragma unroll
        for (int u = 0; u < DEPTH3D_CHUNK; u++) ov[u] = k0 + u < nz ? hn[p + (k0 + u) * plane] : 0.0;
#pragma unroll
        for (int u = 0; u < DEPTH3D_CHUNK; u++) {
            const int k = k0 + u;
            if (k >= nz) break;
            const long long q = p + k * plane;
            const double o = ov[u];
            ho[q] = o;
            double n = o;
            if (m) {
                n = a.dga[k] * D;
                hn[q] = n;
            }
            if (role == 1) {
                const double hh = getm_half(o + n);
                a.hhalf[q] = hh;
                if (i >= 1) a.hnuu[q - 1] = hh;
                if (j >= 1) a.hnvv[q - nx] = hh;
            }
            if (m) sw.level(k, q, plane, H, n, zc, zf);
        }
    }
    if (role == 1 && m && a.depth) t2cd_column(plane, nz, p, a.hnt, a.depth);
}

// c_vertical_advection_to_sources (wrapper.F90:447-485): first-order upstream
// fluxes of c between the levels of a column (for sinking or floating, with
// the vertical velocity w at the layer centres, positive upwards, levels
// ordered surface to bottom), added to the source term s: at interface
// k | k+1 of two wet levels the flux upward * (w_k + w_k+1) / 2 times the
// upstream c leaves level k and enters level k+1, in level order.  Nothing
// changes when w is zero at every interior point (the routine returns
// early then): a first kernel reduces that test into a flag.
__global__ void vadv_sources_active_kernel(int nx, int ny, int nz, int halox, int haloy, const double* w, int* flag)
{
    const long long plane = (long long)nx * ny;
    const long long n = plane * nz;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const long long c = p % plane;
        const int j = (int)(c / nx), i = (int)(c - (long long)j * nx);
        if (i >= halox && i < nx - halox && j >= haloy && j < ny - haloy && w[p] != 0.0) {
            *flag = 1;  // any writer: all write 1
            return;
        }
    }
}

__global__ void vadv_sources_kernel(int nx, int ny, int nz, int halox, int haloy, const int* mask, const double* c,
                                    const double* w, const double* h, double* s, const int* flag)
{
    if (*flag == 0) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y + haloy;
    if (i < halox || i >= nx - halox || j >= ny - haloy) return;
    const long long plane = (long long)nx * ny;
    const long long p = (long long)j * nx + i;
    const double upward = -1.0;  // levels ordered surface to bottom
    for (int k = 0; k < nz - 1; k++) {
        const long long a = p + k * plane, b = a + plane;
        if (mask[a] == 1 && mask[b] == 1) {
            const double local_w = upward * 0.5 * (w[a] + w[b]);
            const double flux = local_w > 0.0 ? local_w * c[a] : local_w * c[b];
            s[a] = s[a] - flux / h[a];
            s[b] = s[b] + flux / h[b];
        }
    }
}

extern "C" int getm_vertical_advection_to_sources(int nx, int ny, int nz, int halox, int haloy, const int* mask,
                                                  const double* c, const double* w, const double* h, double* s,
                                                  int* work, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || halox < 0 || haloy < 0 || 2 * halox >= nx || 2 * haloy >= ny)
        return GETM_ERR_ARG;
    if (!mask || !c || !w || !h || !s || !work) return GETM_ERR_ARG;
    if (cudaMemsetAsync(work, 0, sizeof(int), stream) != cudaSuccess) return GETM_ERR_CUDA;
    const long long n = (long long)nx * ny * nz;
    const int blocks = (int)(getm_div_up(n, 256) < 4096 ? getm_div_up(n, 256) : 4096);
    vadv_sources_active_kernel<<<blocks, 256, 0, stream>>>(nx, ny, nz, halox, haloy, w, work);
    GETM_CHECK_LAUNCH();
    vadv_sources_kernel<<<dim3(getm_div_up(nx, 128), ny - 2 * haloy), 128, 0, stream>>>(nx, ny, nz, halox, haloy,
                                                                                      mask, c, w, h, s, work);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// c_update_gvc (wrapper.F90:567-600): general vertical coordinates, layer
// thicknesses D (dbeta_k + alpha (dsigma - dbeta_k)) where the mask is
// non-zero, with alpha = (min(Dgamma / D, 1) dsigma - dbeta_kk) /
// (dsigma - dbeta_kk) giving the reference layer kk (1-based) the thickness
// min(Dgamma, D) dsigma.
__global__ void update_gvc_kernel(int nx, int ny, int nz, double dsigma, const double* dbeta, double Dgamma, int kk,
                                  const double* D, const int* mask, double* h)
{
    const long long plane = (long long)nx * ny;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= plane) return;
    if (mask[p] == 0) return;
    const double Dp = D[p], db = dbeta[kk - 1];
    const double alpha = (fmin(Dgamma / Dp, 1.0) * dsigma - db) / (dsigma - db);
    for (int k = 0; k < nz; k++) h[p + k * plane] = Dp * (dbeta[k] + alpha * (dsigma - dbeta[k]));
}

extern "C" int getm_update_gvc(int nx, int ny, int nz, double dsigma, const double* dbeta, double Dgamma, int kk,
                               const double* D, const int* mask, double* h, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || kk < 1 || kk > nz) return GETM_ERR_ARG;
    if (!dbeta || !D || !mask || !h) return GETM_ERR_ARG;
    update_gvc_kernel<<<getm_div_up((long long)nx * ny, 128), 128, 0, stream>>>(nx, ny, nz, dsigma, dbeta, Dgamma, kk,
                                                                                  D, mask, h);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
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
    depth_3d_column_kernel<<<dim3(getm_div_up((long long)(nx + 1) * (ny + 1), 128), 4), 128, 0, stream>>>(a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}
