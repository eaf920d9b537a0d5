// Open-boundary conditions and mirroring for sm_103a.
//
// Reference: python/pygetm/open_boundaries.py (ZeroGradient :338-356,
// Clamped :358-375, Flather :377-416, Sponge :195-336, mirroring :848-917
// with core.Array.mirror python/pygetm/core.py:723-728) as driven by
// simulation.py:1160-1168 (tracers), :1252-1257 (elevation), :1545-1550
// (depths) and momentum.py:679, :699, :1212 (transports).
//
// A boundary has a few hundred to a few thousand points, so one thread per
// point (per level for 3D fields).  The reference updates its boundaries one
// after the other; a zero-gradient point next to a corner reads a point of
// another boundary, so the caller launches one boundary (a contiguous range
// of the point tables) at a time, in the reference's order.
#include <math.h>

#include "getm_common.cuh"

#define OB_THREADS 128

namespace {

__device__ __forceinline__ double np_maximum(double lo, double x) { return isnan(x) ? x : fmax(lo, x); }

// elevation at boundary points start..stop-1 (open_boundaries.py:338-416),
// clipped to its minimum Dmin - H (simulation.py:580-582)
__global__ void ob_elevation_kernel(int start, int stop, int nx, const int* bi, const int* bj, const int* type,
                                    const int* di, const int* dj, const int* side, const double* sign,
                                    const double* H, const double* Dclip, const double* U, const double* V,
                                    const double* z_ext, const double* flow_ext, double Dmin, double* z)
{
    const int p = start + blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= stop) return;
    const long long q = (long long)bj[p] * nx + bi[p];
    double v;
    switch (type[p]) {
    case 1:  // ZERO_GRADIENT
        v = z[(long long)(bj[p] + dj[p]) * nx + (bi[p] + di[p])];
        break;
    case 3:  // CLAMPED
        v = z_ext[p];
        break;
    default: {  // FLATHER_ELEV (4), FLATHER_TRANSPORT (-4)
        // transport at the velocity point just inside (extract_uv_in, :149-152)
        double tp;
        switch (side[p]) {
        case 1: tp = U[q]; break;       // WEST: U(j, l)
        case 3: tp = U[q - 1]; break;   // EAST: U(j, l-1)
        case 4: tp = V[q]; break;       // SOUTH: V(l, i)
        default: tp = V[q - nx]; break; // NORTH: V(l-1, i)
        }
        const double D = Dclip[q];
        const double ext = type[p] == 4 ? flow_ext[p] * D : flow_ext[p];
        v = z_ext[p] - sign[p] * (tp - ext) / sqrt(D * GETM_G);
        break;
    }
    }
    z[q] = np_maximum(Dmin - H[q], v);
}

// tracer values at boundary points start..stop-1 for every level and tracer
// of the batch (ZeroGradient, Clamped; Sponge also relaxes the n points
// inward: v += sp_m (bdy - v), sp_m = ((n - m) / (n + 1))^2, only where the
// mask is 1, open_boundaries.py:235-336 without flow-dependent relaxation)
template <typename T>
struct ObTracerArgs {
    int start, stop, nx, nz, nsponge;
    long long plane;
    const int *bi, *bj, *type, *di, *dj, *mask;
    int ntracer;
    T* var[16];
    const T* bdy[16];  // (nz, np) prescribed values per tracer
    int np;
};

template <typename T>
__global__ void ob_tracer_kernel(ObTracerArgs<T> a)
{
    const int p = a.start + blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (p >= a.stop || k >= a.nz) return;
    const long long q = (long long)a.bj[p] * a.nx + a.bi[p] + k * a.plane;
    for (int t = 0; t < a.ntracer; t++) {
        T* f = a.var[t];
        const int ty = a.type[p];
        if (ty == 1) {
            f[q] = f[q + (long long)a.dj[p] * a.nx + a.di[p]];
        } else {
            const T b = a.bdy[t][(long long)k * a.np + p];
            f[q] = b;
            if (ty == 5) {
                for (int m = 0; m < a.nsponge; m++) {
                    const long long o = (long long)(m + 1) * ((long long)a.dj[p] * a.nx + a.di[p]);
                    const long long q2 = (long long)a.bj[p] * a.nx + a.bi[p] + o;  // 2D index of the sponge point
                    if (a.mask[q2] != 1) continue;
                    const T r = (T)(a.nsponge - m) / (T)(a.nsponge + 1);
                    f[q + o] = f[q + o] + (r * r) * (b - f[q + o]);
                }
            }
        }
    }
}

// core.Array.mirror: field[tgt] = field[src] for n pairs of flat 2D indices
// and nlev levels, with numpy's fancy-assignment semantics (every source is
// read before any target is written: a point can be the target of one pair
// and the source of another), hence a gather and a scatter launch.
template <typename T>
__global__ void mirror_gather_kernel(int n, const int* src, int nlev, long long plane, const T* field, T* work)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (p >= n || k >= nlev) return;
    work[(long long)k * n + p] = field[src[p] + k * plane];
}

template <typename T>
__global__ void mirror_scatter_kernel(int n, const int* tgt, int nlev, long long plane, const T* work, T* field)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (p >= n || k >= nlev) return;
    field[tgt[p] + k * plane] = work[(long long)k * n + p];
}

// Depths at the velocity points just outside boundaries: z_T_half.mirror(z_U)
// followed by elevation2depth and alpha there (simulation.py:1545-1552)
__global__ void ob_depth_kernel(int n, const int* srcT, const int* tgt, const double* z, const double* zo,
                                const double* Hv, const int* mv, double Dmin, double twoDmin, double ialpha,
                                double* work, double* D, double* alpha)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int s = srcT[p], t = tgt[p];
    const double zh = (zo[s] + z[s]) * 0.5;
    work[t] = zh;
    if (mv[t] != 0) {
        const double d = fmax(Hv[t] + zh, Dmin);
        D[t] = d;
        alpha[t] = fmax(0.0, fmin(1.0, (d - twoDmin) * ialpha));
    }
}

}  // namespace

extern "C" int getm_open_boundary_elevation(int start, int stop, int nx, const int* i, const int* j,
                                            const int* type, const int* di, const int* dj, const int* side,
                                            const double* inflow_sign, const double* H, const double* Dclip,
                                            const double* U, const double* V, const double* z_ext,
                                            const double* flow_ext, double Dmin, double* z, cudaStream_t stream)
{
    if (start < 0 || stop < start || nx < 1) return GETM_ERR_ARG;
    if (stop == start) return GETM_OK;
    const void* ptrs[] = {i, j, type, di, dj, side, inflow_sign, H, Dclip, U, V, z_ext, flow_ext, z};
    for (const void* q : ptrs)
        if (!q) return GETM_ERR_ARG;
    ob_elevation_kernel<<<getm_div_up(stop - start, OB_THREADS), OB_THREADS, 0, stream>>>(
        start, stop, nx, i, j, type, di, dj, side, inflow_sign, H, Dclip, U, V, z_ext, flow_ext, Dmin, z);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

template <typename T>
static int ob_tracer_impl(int start, int stop, int np, int nx, int ny, int nz, int nsponge, const int* i,
                          const int* j, const int* type, const int* di, const int* dj, const int* mask, int ntracer,
                          T* const* vars, const T* const* bdy, cudaStream_t stream)
{
    if (start < 0 || stop < start || stop > np || nx < 1 || ny < 1 || nz < 1 || nsponge < 0 || ntracer < 0 ||
        ntracer > 16)
        return GETM_ERR_ARG;
    if (stop == start || ntracer == 0) return GETM_OK;
    if (!i || !j || !type || !di || !dj || !mask || !vars || !bdy) return GETM_ERR_ARG;
    ObTracerArgs<T> a;
    a.start = start; a.stop = stop; a.nx = nx; a.nz = nz; a.nsponge = nsponge; a.np = np;
    a.plane = (long long)nx * ny;
    a.bi = i; a.bj = j; a.type = type; a.di = di; a.dj = dj; a.mask = mask; a.ntracer = ntracer;
    for (int t = 0; t < ntracer; t++) {
        if (!vars[t] || !bdy[t]) return GETM_ERR_ARG;
        a.var[t] = vars[t];
        a.bdy[t] = bdy[t];
    }
    dim3 grid(getm_div_up(stop - start, OB_THREADS), nz);
    ob_tracer_kernel<T><<<grid, OB_THREADS, 0, stream>>>(a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_open_boundary_tracers(int start, int stop, int np, int nx, int ny, int nz, int nsponge,
                                          const int* i, const int* j, const int* type, const int* di,
                                          const int* dj, const int* mask, int ntracer, double* const* vars,
                                          const double* const* bdy, cudaStream_t stream)
{
    return ob_tracer_impl<double>(start, stop, np, nx, ny, nz, nsponge, i, j, type, di, dj, mask, ntracer, vars, bdy,
                                  stream);
}

extern "C" int getm_open_boundary_tracers_f32(int start, int stop, int np, int nx, int ny, int nz, int nsponge,
                                              const int* i, const int* j, const int* type, const int* di,
                                              const int* dj, const int* mask, int ntracer, float* const* vars,
                                              const float* const* bdy, cudaStream_t stream)
{
    return ob_tracer_impl<float>(start, stop, np, nx, ny, nz, nsponge, i, j, type, di, dj, mask, ntracer, vars, bdy,
                                 stream);
}

template <typename T>
static int mirror_impl(int n, const int* src, const int* tgt, int nlev, long long plane, T* field, T* work,
                       cudaStream_t stream)
{
    if (n < 0 || nlev < 1 || plane < 1) return GETM_ERR_ARG;
    if (n == 0) return GETM_OK;
    if (!src || !tgt || !field || !work) return GETM_ERR_ARG;
    dim3 grid(getm_div_up(n, OB_THREADS), nlev);
    mirror_gather_kernel<T><<<grid, OB_THREADS, 0, stream>>>(n, src, nlev, plane, field, work);
    GETM_CHECK_LAUNCH();
    mirror_scatter_kernel<T><<<grid, OB_THREADS, 0, stream>>>(n, tgt, nlev, plane, work, field);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_mirror(int n, const int* src, const int* tgt, int nlev, long long plane, double* field,
                           double* work, cudaStream_t stream)
{
    return mirror_impl<double>(n, src, tgt, nlev, plane, field, work, stream);
}

extern "C" int getm_mirror_f32(int n, const int* src, const int* tgt, int nlev, long long plane, float* field,
                               float* work, cudaStream_t stream)
{
    return mirror_impl<float>(n, src, tgt, nlev, plane, field, work, stream);
}

extern "C" int getm_open_boundary_depth(int n, const int* srcT, const int* tgt, const double* z, const double* zo,
                                        const double* H, const int* mask, double Dmin, double Dcrit, double* work,
                                        double* D, double* alpha, cudaStream_t stream)
{
    if (n < 0) return GETM_ERR_ARG;
    if (n == 0) return GETM_OK;
    if (!srcT || !tgt || !z || !zo || !H || !mask || !work || !D || !alpha) return GETM_ERR_ARG;
    ob_depth_kernel<<<getm_div_up(n, OB_THREADS), OB_THREADS, 0, stream>>>(
        n, srcT, tgt, z, zo, H, mask, Dmin, 2 * Dmin, 1.0 / (Dcrit - 2 * Dmin), work, D, alpha);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}
