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

#include "split2d_ops.cuh"

#include <type_traits>

#define S2_THREADS 128

namespace {

template <int BY, bool MIXED>
__global__ void __launch_bounds__(UD_BX * BY) update_depth_2d_kernel(DepthArgs a)
{
    __shared__ double szh[BY + 2][UD_BX + 2];
    update_depth_2d_tile<BY, MIXED>(a, blockIdx.x, blockIdx.y, threadIdx.x, threadIdx.y, szh);
}

template <typename C>
__global__ void __launch_bounds__(S2_THREADS) momentum_2d_velocities_kernel(VelArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= a.nx || j >= a.ny) return;
    momentum_2d_velocities_point<C>(a, i, j);
}

template <typename C>
__global__ void __launch_bounds__(S2_THREADS) momentum_2d_friction_kernel(FricArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= a.nx || j >= a.ny) return;
    momentum_2d_friction_point<C>(a, i, j);
}

template <typename C>
__global__ void __launch_bounds__(S2_THREADS) coriolis_2d_kernel(int nx, int ny, int ioff, int joff,
                                                                  const double* src, const double* cor,
                                                                  double* out, int negate)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= nx || j >= ny) return;
    coriolis_2d_point<C>(nx, ny, ioff, joff, src, cor, out, negate, i, j);
}

// Momentum.coriolis for 3D transports (momentum.py:1127-1148, DEFAULT
// scheme): interp_xy of every layer to the other velocity grid, times f,
// negated for the V equation, as one launch.  T: storage and arithmetic
// (float in the mixed form: f narrowed on the integer pipe).
template <typename T>
__global__ void __launch_bounds__(S2_THREADS) coriolis_3d_kernel(int nx, int ny, int ioff, int joff,
                                                                  const T* __restrict__ src,
                                                                  const double* __restrict__ cor,
                                                                  T* __restrict__ out, int negate)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    const long long off = (long long)blockIdx.z * nx * ny;
    if (i >= nx || j >= ny) return;
    const long long p = (long long)j * nx + i;
    const int si = i - ioff, sj = j - joff;
    T v;
    if (si >= 0 && sj >= 0 && si <= nx - 2 && sj <= ny - 2) {
        const long long q = off + (long long)sj * nx + si;
        v = T(0.25) * (src[q] + src[q + 1] + src[q + nx] + src[q + nx + 1]);
    } else {
        v = out[off + p];
    }
    if constexpr (std::is_same<T, double>::value) v = v * cor[p];
    else v = v * getm_d2f_approx(cor[p]);
    out[off + p] = negate ? -v : v;
}

// Inputs of the 3D momentum advection (momentum.py:989-1003): the velocities
// interpolated to the UU, UV, VU, VV grids (uk -> UU and vk -> UV by
// interp_x, uk -> VU and vk -> VV by interp_y), ww interpolated to U and V,
// and the advected copies of uk and vk, in one launch; grid (x, ny, nz + 1),
// the top level holds only the interface values of ww.  Each target keeps
// its previous value where the interpolation does not write (as interp_x/y).
template <typename T>
struct Mom3DIn {
    int nx, ny, nz;
    long long plane;
    const T *uk, *vk, *ww;
    T *uua, *uva, *vua, *vva, *wwu, *wwv, *advpk, *advqk;
};

template <typename T>
__global__ void __launch_bounds__(S2_THREADS) momentum_3d_inputs_kernel(Mom3DIn<T> a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= a.nx) return;
    const long long p = (long long)k * a.plane + (long long)j * a.nx + i;
    const bool ex = i < a.nx - 1, ey = j < a.ny - 1;
    if (ex) interp_pair_point<T>(a.ww, a.wwu, p, 1, 0);
    if (ey) interp_pair_point<T>(a.ww, a.wwv, p, a.nx, 0);
    if (k == a.nz) return;
    if (ex) {
        interp_pair_point<T>(a.uk, a.uua, p, 1, 0);
        interp_pair_point<T>(a.vk, a.uva, p, 1, 0);
    }
    if (ey) {
        interp_pair_point<T>(a.uk, a.vua, p, a.nx, 0);
        interp_pair_point<T>(a.vk, a.vva, p, a.nx, 0);
    }
    a.advpk[p] = a.uk[p];
    a.advqk[p] = a.vk[p];
}

__global__ void __launch_bounds__(S2_THREADS) advance_2d_transport_mixed_kernel(int nx, int ny, int halox, int haloy,
                                                                                 Transport2DArgs a, double dt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i < halox || i >= nx - halox || j < haloy || j >= ny - haloy) return;
    transport_2d_mixed_point(a, dt, (long long)j * nx + i);
}

__global__ void accumulate_2d_kernel(long long n, const double* U, const double* V, double* Uc, double* Vc)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    accumulate_2d_point(U, V, Uc, Vc, p);
}

__global__ void __launch_bounds__(S2_THREADS) surface_elevation_fused_kernel(
    int nx, int ny, int halox, int haloy, const int* mask, const double* dyu, const double* dxv,
    const double* iarea, double* z, double* zo, const double* U, const double* V, const double* fwf, double dt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= nx || j >= ny) return;
    surface_elevation_fused_point(nx, ny, halox, haloy, mask, dyu, dxv, iarea, z, zo, U, V, fwf, dt, i, j);
}

}  // namespace

static inline dim3 plane_grid(int nx, int ny) { return dim3(getm_div_up(nx, S2_THREADS), ny); }

template <bool MIXED>
static int update_depth_2d_impl(int nx, int ny, double Dmin, double Dcrit, const double* z, const double* zo,
                                const double* HT, const double* HU, const double* HV, const double* HX, const int* mT,
                                const int* mU, const int* mV, const int* mX, double* DT, double* DclipT,
                                double* workT, double* workU, double* DU, double* alphaU, double* workV, double* DV,
                                double* alphaV, double* workX, double* DX, double* DUU, double* DVV, double* DUV,
                                double* DVU, cudaStream_t stream)
{
    if (nx < 2 || ny < 2) return GETM_ERR_ARG;
    const void* ptrs[] = {z, zo, HT, HU, HV, HX, mT, mU, mV, mX, DT, DclipT, workT, workU, DU, alphaU,
                          workV, DV, alphaV, workX, DX, DUU, DVV, DUV, DVU};
    for (const void* q : ptrs)
        if (!q) return GETM_ERR_ARG;
    DepthArgs a{nx, ny, Dmin, Dcrit, 1.0 / (Dcrit - 2 * Dmin), z, zo, HT, HU, HV, HX, mT, mU, mV, mX, DT, DclipT,
                workT, workU, DU, alphaU, workV, DV, alphaV, workX, DX, DUU, DVV, DUV, DVU};
    constexpr int BY = 4;
    dim3 block(UD_BX, BY);
    dim3 grid(getm_div_up(nx + 1, UD_BX), getm_div_up(ny + 1, BY));
    update_depth_2d_kernel<BY, MIXED><<<grid, block, 0, stream>>>(a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_update_depth_2d(int nx, int ny, double Dmin, double Dcrit, const double* z, const double* zo,
                                    const double* HT, const double* HU, const double* HV, const double* HX,
                                    const int* mT, const int* mU, const int* mV, const int* mX, double* DT,
                                    double* DclipT, double* workT, double* workU, double* DU, double* alphaU,
                                    double* workV, double* DV, double* alphaV, double* workX, double* DX,
                                    double* DUU, double* DVV, double* DUV, double* DVU, cudaStream_t stream)
{
    return update_depth_2d_impl<false>(nx, ny, Dmin, Dcrit, z, zo, HT, HU, HV, HX, mT, mU, mV, mX, DT, DclipT, workT,
                                       workU, DU, alphaU, workV, DV, alphaV, workX, DX, DUU, DVV, DUV, DVU, stream);
}

extern "C" int getm_update_depth_2d_mixed(int nx, int ny, double Dmin, double Dcrit, const double* z,
                                          const double* zo, const double* HT, const double* HU, const double* HV,
                                          const double* HX, const int* mT, const int* mU, const int* mV,
                                          const int* mX, double* DT, double* DclipT, double* workT, double* workU,
                                          double* DU, double* alphaU, double* workV, double* DV, double* alphaV,
                                          double* workX, double* DX, double* DUU, double* DVV, double* DUV,
                                          double* DVU, cudaStream_t stream)
{
    return update_depth_2d_impl<true>(nx, ny, Dmin, Dcrit, z, zo, HT, HU, HV, HX, mT, mU, mV, mX, DT, DclipT, workT,
                                      workU, DU, alphaU, workV, DV, alphaV, workX, DX, DUU, DVV, DUV, DVU, stream);
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

template <typename C>
static int coriolis_impl(int nx, int ny, int ioffset, int joffset, const double* src, const double* cor, double* out,
                         int negate, cudaStream_t stream)
{
    if (nx < 2 || ny < 2 || !src || !cor || !out || ioffset < 0 || ioffset > 1 || joffset < 0 || joffset > 1)
        return GETM_ERR_ARG;
    coriolis_2d_kernel<C><<<plane_grid(nx, ny), S2_THREADS, 0, stream>>>(nx, ny, ioffset, joffset, src, cor, out,
                                                                         negate);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_coriolis_2d(int nx, int ny, int ioffset, int joffset, const double* src, const double* cor,
                                double* out, int negate, cudaStream_t stream)
{
    return coriolis_impl<double>(nx, ny, ioffset, joffset, src, cor, out, negate, stream);
}

extern "C" int getm_coriolis_2d_mixed(int nx, int ny, int ioffset, int joffset, const double* src,
                                      const double* cor, double* out, int negate, cudaStream_t stream)
{
    return coriolis_impl<float>(nx, ny, ioffset, joffset, src, cor, out, negate, stream);
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
    Transport2DArgs a{mask, alpha, D, dp, taus, cor, adv, diff, damp, SA, SB, SD, SF, r, U};
    advance_2d_transport_mixed_kernel<<<plane_grid(nx, ny), S2_THREADS, 0, stream>>>(nx, ny, halox, haloy, a, dt);
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

template <typename T>
static int coriolis_3d_impl(int nx, int ny, int nz, int ioffset, int joffset, const T* src, const double* cor, T* out,
                            int negate, cudaStream_t stream)
{
    if (nx < 2 || ny < 2 || nz < 1 || !src || !cor || !out || ioffset < 0 || ioffset > 1 || joffset < 0 || joffset > 1)
        return GETM_ERR_ARG;
    dim3 grid(getm_div_up(nx, S2_THREADS), ny, nz);
    coriolis_3d_kernel<T><<<grid, S2_THREADS, 0, stream>>>(nx, ny, ioffset, joffset, src, cor, out, negate);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// Momentum.coriolis, ESPELID scheme (momentum.py:1136-1142), 2D or 3D: the
// transport is divided by sqrt(D) of its own grid (1 on land) before the
// interp_xy to the other velocity grid, and the result is multiplied by
// sqrt(D) of the target grid on water points, then by f and negated for the
// V equation.  D: water depth (2D) or layer thickness (3D) of each grid.
// Target points outside the interpolation range keep their old value, as
// interp leaves them (then scaled like the rest).  On land points of the
// target the reference multiplies by an unset value (np.sqrt with where=
// and no out=); here the sqrt(D) factor is left out there.  The transport
// update never reads the term on land.  FP64 arithmetic, T storage.
template <typename T>
__global__ void __launch_bounds__(S2_THREADS) coriolis_espelid_kernel(
    int nx, int ny, int ioff, int joff, const T* __restrict__ src, const double* __restrict__ Din,
    const int* __restrict__ mask_in, const double* __restrict__ Dout, const int* __restrict__ mask_out,
    const double* __restrict__ cor, T* __restrict__ out, int negate)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    const long long off = (long long)blockIdx.z * nx * ny;
    if (i >= nx || j >= ny) return;
    const long long p = (long long)j * nx + i;
    const int si = i - ioff, sj = j - joff;
    double v;
    if (si >= 0 && sj >= 0 && si <= nx - 2 && sj <= ny - 2) {
        const long long q = (long long)sj * nx + si;
        auto scaled = [&](long long r) {
            const double s = mask_in[r] != 0 ? sqrt(Din[off + r]) : 1.0;
            return (double)src[off + r] / s;
        };
        v = 0.25 * (scaled(q) + scaled(q + 1) + scaled(q + nx) + scaled(q + nx + 1));
    } else {
        v = (double)out[off + p];
    }
    if (mask_out[p] != 0) v = v * sqrt(Dout[off + p]);
    v = v * cor[p];
    out[off + p] = (T)(negate ? -v : v);
}

template <typename T>
static int coriolis_espelid_impl(int nx, int ny, int nz, int ioffset, int joffset, const T* src, const double* Din,
                                 const int* mask_in, const double* Dout, const int* mask_out, const double* cor,
                                 T* out, int negate, cudaStream_t stream)
{
    if (nx < 2 || ny < 2 || nz < 1 || !src || !Din || !mask_in || !Dout || !mask_out || !cor || !out ||
        ioffset < 0 || ioffset > 1 || joffset < 0 || joffset > 1)
        return GETM_ERR_ARG;
    dim3 grid(getm_div_up(nx, S2_THREADS), ny, nz);
    coriolis_espelid_kernel<T><<<grid, S2_THREADS, 0, stream>>>(nx, ny, ioffset, joffset, src, Din, mask_in, Dout,
                                                                mask_out, cor, out, negate);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_coriolis_espelid(int nx, int ny, int nz, int ioffset, int joffset, const double* src,
                                     const double* Din, const int* mask_in, const double* Dout,
                                     const int* mask_out, const double* cor, double* out, int negate,
                                     cudaStream_t stream)
{
    return coriolis_espelid_impl<double>(nx, ny, nz, ioffset, joffset, src, Din, mask_in, Dout, mask_out, cor, out,
                                         negate, stream);
}

extern "C" int getm_coriolis_espelid_f32(int nx, int ny, int nz, int ioffset, int joffset, const float* src,
                                         const double* Din, const int* mask_in, const double* Dout,
                                         const int* mask_out, const double* cor, float* out, int negate,
                                         cudaStream_t stream)
{
    return coriolis_espelid_impl<float>(nx, ny, nz, ioffset, joffset, src, Din, mask_in, Dout, mask_out, cor, out,
                                        negate, stream);
}

extern "C" int getm_coriolis_3d(int nx, int ny, int nz, int ioffset, int joffset, const double* src, const double* cor,
                                double* out, int negate, cudaStream_t stream)
{
    return coriolis_3d_impl<double>(nx, ny, nz, ioffset, joffset, src, cor, out, negate, stream);
}

extern "C" int getm_coriolis_3d_f32(int nx, int ny, int nz, int ioffset, int joffset, const float* src,
                                    const double* cor, float* out, int negate, cudaStream_t stream)
{
    return coriolis_3d_impl<float>(nx, ny, nz, ioffset, joffset, src, cor, out, negate, stream);
}

template <typename T>
static int momentum_3d_inputs_impl(int nx, int ny, int nz, const T* uk, const T* vk, const T* ww, T* uua, T* uva,
                                   T* vua, T* vva, T* wwu, T* wwv, T* advpk, T* advqk, cudaStream_t stream)
{
    if (nx < 2 || ny < 2 || nz < 1) return GETM_ERR_ARG;
    const void* ptrs[] = {uk, vk, ww, uua, uva, vua, vva, wwu, wwv, advpk, advqk};
    for (const void* q : ptrs)
        if (!q) return GETM_ERR_ARG;
    Mom3DIn<T> a{nx, ny, nz, (long long)nx * ny, uk, vk, ww, uua, uva, vua, vva, wwu, wwv, advpk, advqk};
    dim3 grid(getm_div_up(nx, S2_THREADS), ny, nz + 1);
    momentum_3d_inputs_kernel<T><<<grid, S2_THREADS, 0, stream>>>(a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_momentum_3d_advection_inputs(int nx, int ny, int nz, const double* uk, const double* vk,
                                                 const double* ww, double* uua, double* uva, double* vua,
                                                 double* vva, double* wwu, double* wwv, double* advpk,
                                                 double* advqk, cudaStream_t stream)
{
    return momentum_3d_inputs_impl<double>(nx, ny, nz, uk, vk, ww, uua, uva, vua, vva, wwu, wwv, advpk, advqk, stream);
}

extern "C" int getm_momentum_3d_advection_inputs_f32(int nx, int ny, int nz, const float* uk, const float* vk,
                                                     const float* ww, float* uua, float* uva, float* vua,
                                                     float* vva, float* wwu, float* wwv, float* advpk,
                                                     float* advqk, cudaStream_t stream)
{
    return momentum_3d_inputs_impl<float>(nx, ny, nz, uk, vk, ww, uua, uva, vua, vva, wwu, wwv, advpk, advqk, stream);
}
