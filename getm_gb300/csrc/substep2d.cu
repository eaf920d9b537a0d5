// One split-explicit 2D substep as one persistent kernel for sm_103a.
//
// A 2D substep of pygetm's Simulation.advance that is not followed by a 3D
// (macro) step (python/pygetm/simulation.py:1033-1304: advance_depth_integrated,
// advance_surface_elevation, update_depth, update_depth_integrated_diagnostics,
// the surface pressure gradient and the wind-stress interpolation) is some
// twenty operations on fields of one horizontal plane.  Launched one by one
// they leave GB300 idle between launches: each reads and writes ~10^5 points,
// a microsecond of work behind several microseconds of launch and drain.
//
// Here one cooperative launch runs the whole substep.  Its blocks (one or
// two per SM, 512 threads) walk through seven phases separated by grid-wide
// barriers; a phase contains operations whose inputs at neighbouring points
// were completed by an earlier phase:
//   1  transport update of the first direction (U or V, alternating)
//   2  Coriolis term from it, then the second direction's update
//   3  Coriolis term from the second, cumulative transports, zo = z and the
//      surface elevation update
//   4  depths (update_depth, 2D part), fwf = pe, wind stress interpolation
//   5  velocities and advection velocities, copies of the depths advected
//      by the momentum advection, surface pressure gradient
//   6  bottom friction, first pass of the U and V momentum advection
//   7  second pass of both, forming each cell's advection term from its
//      transport change as the pass finishes the cell (reconstruct)
// Every operation is the same device function the separate kernels run
// (split2d_ops.cuh, advection_passes.cuh), so results are bitwise the same.
//
// The barrier is a counter and a generation word in global memory.  Its wait
// is bounded: after about a second it sets the error word, every block
// returns, and later launches return at once until the host clears the word.
#include <string.h>

#include <mutex>
#include <type_traits>

#include "advection_passes.cuh"
#include "split2d_ops.cuh"

namespace {

constexpr int SS_BY = 16;
constexpr int SS_THREADS = 32 * SS_BY;
constexpr unsigned SS_SPIN_LIMIT = 1u << 22;

__device__ __forceinline__ int div_up(int a, int b) { return (a + b - 1) / b; }

struct SubstepArgs {
    int nx, ny, halox, haloy;
    int ufirst, accumulate, friction;
    double dt, idt;
    double* time;
    Transport2DArgs tr[2];       // [0]: U, [1]: V
    double* cor_out[2];          // Coriolis terms corU, corV (read by tr[].cor)
    const double* corf[2];       // Coriolis parameter on U, V
    double *Ucum, *Vcum;
    const int* mT;
    const double *dyU, *dxV, *iareaT;
    double *z, *zo, *fwf;
    const double* pe;
    DepthArgs depth;
    VelArgs vel;
    FricArgs fric;
    SpgArgs spg;
    const double *taux, *tauy;
    double *tausx, *tausy;
    Advection2DPasses adv[2];    // momentum advection of U and V
    const double* Dsrc[2];       // U.D, V.D
    double* advD[2];             // the advections' thickness arrays
    double* advvar[2];           // advU, advV
    const double* Uo[2];         // U, V
    unsigned* sync;              // [0] barrier arrivals, [1] blocks done, [2] error
};

static_assert(SS_BY == GETM_V_BY && SS_BY == HY_BY, "the y passes run on the kernel's 32 x 16 blocks");

union SubstepSmem {
    double szh[SS_BY + 2][UD_BX + 2];
    struct {
        double sQ[GETM_V_BY][32];
        double sF[GETM_V_BY][32];
    } y;
    YIncSmem<double> yi;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" : : "l"(p), "r"(v) : "memory");
}

// Grid-wide barrier k of a launch: thread 0 of every block adds one arrival
// and waits until the count reaches k blocks per block; false when the wait
// gave up or another block reported an error (the caller returns).  The
// count only grows during a launch; the last block to leave the kernel
// resets it (grid_exit) for the next launch on the stream.  Ordering: the
// block barrier orders the block's writes before thread 0's release
// arrival, and thread 0's acquire load followed by the block barrier orders
// the other blocks' writes before every thread's later reads.
__device__ __forceinline__ bool grid_barrier(unsigned* sync, unsigned& target, int& s_ok)
{
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        target += gridDim.x;
        red_release_add(&sync[0], 1u);
        int ok = 1;
        unsigned it = 0;
        while (ld_acquire(&sync[0]) < target) {
            if (++it > SS_SPIN_LIMIT) {
                atomicExch(&sync[2], 1u);
                ok = 0;
                break;
            }
            if ((it & 255u) == 0 && ld_acquire(&sync[2]) != 0) {  // another block gave up
                ok = 0;
                break;
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

__device__ __forceinline__ void grid_exit(unsigned* sync)
{
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        __threadfence();
        if (atomicAdd(&sync[1], 1u) == gridDim.x - 1) {
            atomicExch(&sync[0], 0u);
            atomicExch(&sync[1], 0u);
        }
    }
}

// One advection pass over the whole plane, distributed over the grid: x
// passes by warps (one row segment each), y passes by blocks (one tile each).
// reconstruct_transport_change (momentum.F90:323-340) of a cell as soon as
// the last advection pass has finished it: un = (un hn - Uo) / dt on rows
// jlo..jhi (the same expression as reconstruct_point)
struct ReconstructEpi {
    double* un;
    const double* Uo;
    double idt;
    int jlo, jhi;
    __device__ __forceinline__ void operator()(long long p, int j, double fn, double hn) const
    {
        if (j < jlo || j > jhi) return;
        un[p] = (fn * hn - Uo[p]) * idt;
    }
};

template <bool MIXED, typename Epi = NoEpi>
__device__ __forceinline__ void advection_pass(const HPassArgs<double>& pa, int dir, SubstepSmem& sm, int tx,
                                               int ty, const Epi& epi = Epi())
{
    if (dir == 1) {
        const int nbx = MIXED ? div_up(pa.nx_ + 1, HX_STRIDE) : div_up(pa.nx_, 32);
        const long long items = (long long)nbx * pa.ny_;
        // equal contiguous runs of row segments per block (every SM busy)
        const long long per = (items + gridDim.x - 1) / gridDim.x;
        const long long wb = (long long)blockIdx.x * per, we = wb + per < items ? wb + per : items;
        for (long long w = wb + ty; w < we; w += SS_BY) {
            const int bx = (int)(w % nbx);
            const long long row = w / nbx;
            if constexpr (MIXED) hpass_x_inc_body<double, Epi>(pa, bx, row, tx, epi);
            else hpass_x_body<double, Epi>(pa, bx, row, tx, epi);
        }
    } else {
        const int nbx = div_up(pa.nx_, 32);
        const int nby = MIXED ? div_up(pa.ny_ + 1, HY_STRIDE) : div_up(pa.ny_, GETM_V_BY);
        for (int t = blockIdx.x; t < nbx * nby; t += gridDim.x) {
            if constexpr (MIXED) hpass_y_inc_body<double, Epi>(pa, t % nbx, t / nbx, 0, tx, ty, sm.yi, epi);
            else hpass_y_body<double, Epi>(pa, t % nbx, t / nbx, 0, tx, ty, sm.y.sQ, sm.y.sF, epi);
            __syncthreads();  // shared memory is reused by the next tile
        }
    }
}

template <bool MIXED>
__device__ __forceinline__ void transport_update(const Transport2DArgs& t, double dt, long long p)
{
    if constexpr (MIXED) transport_2d_mixed_point(t, dt, p);
    else transport_2d_point(t, dt, p);
}

// Coriolis term on the other velocity grid from the transport of direction
// d (momentum.py:1127-1148): U -> V with offsets (1, 0), negated; V -> U
// with offsets (0, 1).
template <typename C>
__device__ __forceinline__ void coriolis_from(const SubstepArgs& a, int d, int i, int j)
{
    const int o = 1 - d;
    coriolis_2d_point<C>(a.nx, a.ny, d == 0 ? 1 : 0, d == 0 ? 0 : 1, a.tr[d].U, a.corf[o], a.cor_out[o], d == 0, i,
                         j);
}

template <bool MIXED>
__global__ void __launch_bounds__(SS_THREADS, MIXED ? 2 : 1) substep_2d_kernel(SubstepArgs a)
{
    using C = typename std::conditional<MIXED, float, double>::type;
    __shared__ SubstepSmem sm;
    __shared__ int s_ok;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int gt = blockIdx.x * SS_THREADS + ty * 32 + tx;
    // pointwise phases: the plane in equal contiguous chunks, one per block,
    // so every SM gets the same number of points (a grid-stride loop over
    // fewer points than threads would leave the last blocks idle and give
    // the first SMs a third more work); consecutive threads take
    // consecutive points
    const int tid = ty * 32 + tx;
    const int nx = a.nx, ny = a.ny;
    const int n = nx * ny;  // < 2^30 (checked by the host)
    const int chunk = (n + (int)gridDim.x - 1) / (int)gridDim.x;
    const int pb = (int)blockIdx.x * chunk, pe = min(pb + chunk, n);
    const int ilo = a.halox, ihi = nx - a.halox - 1, jlo = a.haloy, jhi = ny - a.haloy - 1;

    unsigned target = 0;  // barrier count to wait for (thread 0)
    if (tx == 0 && ty == 0) s_ok = ld_acquire(&a.sync[2]) == 0;
    __syncthreads();
    if (!s_ok) return;

    const int d1 = a.ufirst ? 0 : 1, d2 = 1 - d1;
    // 1: first transport update
    for (int p = pb + tid; p < pe; p += SS_THREADS) {
        const int j = p / nx, i = p - j * nx;
        if (i >= ilo && i <= ihi && j >= jlo && j <= jhi) transport_update<MIXED>(a.tr[d1], a.dt, p);
    }
    if (!grid_barrier(a.sync, target, s_ok)) return grid_exit(a.sync);
    // 2: Coriolis from the first, second transport update
    for (int p = pb + tid; p < pe; p += SS_THREADS) {
        const int j = p / nx, i = p - j * nx;
        coriolis_from<C>(a, d1, i, j);
        if (i >= ilo && i <= ihi && j >= jlo && j <= jhi) transport_update<MIXED>(a.tr[d2], a.dt, p);
    }
    if (!grid_barrier(a.sync, target, s_ok)) return grid_exit(a.sync);
    // 3: Coriolis from the second, cumulative transports, surface elevation
    for (int p = pb + tid; p < pe; p += SS_THREADS) {
        const int j = p / nx, i = p - j * nx;
        coriolis_from<C>(a, d2, i, j);
        if (a.accumulate) accumulate_2d_point(a.tr[0].U, a.tr[1].U, a.Ucum, a.Vcum, p);
        surface_elevation_fused_point(nx, ny, a.halox, a.haloy, a.mT, a.dyU, a.dxV, a.iareaT, a.z, a.zo,
                                      a.tr[0].U, a.tr[1].U, a.fwf, a.dt, i, j);
    }
    if (!grid_barrier(a.sync, target, s_ok)) return grid_exit(a.sync);
    // 4: depths; fwf = pe; wind stress on U and V (interp_x/y, offset 0)
    {
        const int ntx = div_up(nx + 1, UD_BX), nty = div_up(ny + 1, SS_BY);
        for (int t = blockIdx.x; t < ntx * nty; t += gridDim.x) {
            update_depth_2d_tile<SS_BY, MIXED>(a.depth, t % ntx, t / ntx, tx, ty, sm.szh);
            __syncthreads();
        }
    }
    for (int p = pb + tid; p < pe; p += SS_THREADS) {
        const int j = p / nx, i = p - j * nx;
        a.fwf[p] = a.pe[p];
        if (i < nx - 1) interp_pair_point<double>(a.taux, a.tausx, p, 1, 0);
        if (j < ny - 1) interp_pair_point<double>(a.tauy, a.tausy, p, nx, 0);
    }
    if (!grid_barrier(a.sync, target, s_ok)) return grid_exit(a.sync);
    // 5: velocities, advected thicknesses, surface pressure gradient
    for (int p = pb + tid; p < pe; p += SS_THREADS) {
        const int j = p / nx, i = p - j * nx;
        momentum_2d_velocities_point<C>(a.vel, i, j);
        a.advD[0][p] = a.Dsrc[0][p];
        a.advD[1][p] = a.Dsrc[1][p];
        if (i >= ilo && i <= ihi && j >= jlo && j <= jhi) spg_point<MIXED>(a.spg, p);
    }
    if (!grid_barrier(a.sync, target, s_ok)) return grid_exit(a.sync);
    // 6: bottom friction; first advection passes
    if (a.friction) {
        for (int p = pb + tid; p < pe; p += SS_THREADS) {
            const int j = p / nx, i = p - j * nx;
            momentum_2d_friction_point<C>(a.fric, i, j);
        }
    }
    advection_pass<MIXED>(a.adv[0].pass[0], a.adv[0].dir[0], sm, tx, ty);
    advection_pass<MIXED>(a.adv[1].pass[0], a.adv[1].dir[0], sm, tx, ty);
    if (!grid_barrier(a.sync, target, s_ok)) return grid_exit(a.sync);
    // 7: second advection passes, each cell's advection term formed as the
    // pass finishes it (reconstruct_transport_change).  The model time moves
    // on only here, after the last barrier: a substep abandoned at a barrier
    // leaves it unchanged (no phase reads it).
    if (gt == 0 && a.time) *a.time = *a.time + a.dt;
    for (int d = 0; d < 2; d++) {
        const ReconstructEpi epi{a.advvar[d], a.Uo[d], a.idt, jlo, jhi};
        advection_pass<MIXED>(a.adv[d].pass[1], a.adv[d].dir[1], sm, tx, ty, epi);
    }
    grid_exit(a.sync);
}

static_assert(sizeof(SubstepArgs) <= 4096, "kernel parameter block");

constexpr int SS_MAX_DEVICES = 64;

// Co-resident blocks of substep_2d_kernel<MIXED> on device `dev` (SMs times
// blocks per SM), queried once per device and kept under a mutex, so host
// threads driving different GPUs each get their own device's count.
template <bool MIXED>
int substep_blocks(int dev, int* blocks)
{
    static int cache[SS_MAX_DEVICES];
    static std::mutex mutex;
    if (dev < 0 || dev >= SS_MAX_DEVICES) return GETM_ERR_ARG;
    std::lock_guard<std::mutex> lock(mutex);
    if (cache[dev] == 0) {
        int sms = 0, coop = 0, per_sm = 0;
        if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
            return GETM_ERR_CUDA;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GETM_ERR_CUDA;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, substep_2d_kernel<MIXED>, SS_THREADS, 0) !=
                cudaSuccess ||
            per_sm < 1)
            return GETM_ERR_CUDA;
        cache[dev] = sms * per_sm;
    }
    *blocks = cache[dev];
    return GETM_OK;
}

template <bool MIXED>
int launch_substep(const SubstepArgs& a, cudaStream_t stream)
{
    int dev = 0, blocks = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GETM_ERR_CUDA;
    if (int rc = substep_blocks<MIXED>(dev, &blocks)) return rc;
    // launch-shape knob: fewer blocks per SM than fit (never more)
    const int per_sm = getm_tune(GETM_TUNE_SUBSTEP_BLOCKS);
    if (per_sm > 0) {
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GETM_ERR_CUDA;
        if (per_sm * sms < blocks) blocks = per_sm * sms;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(32, SS_BY);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, substep_2d_kernel<MIXED>, a) != cudaSuccess) return GETM_ERR_CUDA;
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

}  // namespace

namespace {

// The kernel's arguments for one domain from its fields and handles; a
// GETM_* status.
int substep_args(SubstepArgs& a, const getm_split2d_fields* f, int nx, int ny, int halox, int haloy, int mixed,
                 int ufirst, int accumulate, int friction, double timestep, double Dmin, double Dcrit,
                 getm_advection* uadv, getm_grid* ugrid, getm_grid* uugrid, getm_grid* uvgrid, int uadv_ufirst,
                 getm_advection* vadv, getm_grid* vgrid, getm_grid* vugrid, getm_grid* vvgrid, int vadv_ufirst)
{
    if (!f || nx < 2 || ny < 2 || halox < 1 || haloy < 1 || !(timestep > 0.0) || !uadv || !vadv) return GETM_ERR_ARG;
    if ((long long)(nx + 1) * (ny + 1) >= (1ll << 30)) return GETM_ERR_ARG;
    const void* ptrs[] = {f->mask_t, f->H_t, f->iarea_t, f->z, f->zo, f->D_t, f->Dclip_t, f->work_t, f->fwf, f->pe,
                          f->sp, f->taux, f->tauy,
                          f->mask_u, f->H_u, f->dy_u, f->idx_u, f->cor_u, f->z0b_u, f->D_u, f->alpha_u, f->work_u,
                          f->U, f->dpdx, f->tausx, f->corU, f->advU, f->diffU, f->dampU, f->SxA, f->SxB, f->SxD,
                          f->SxF, f->ru, f->u1, f->Ucum, f->advD_u, f->uua, f->uva,
                          f->mask_v, f->H_v, f->dx_v, f->idy_v, f->cor_v, f->z0b_v, f->D_v, f->alpha_v, f->work_v,
                          f->V, f->dpdy, f->tausy, f->corV, f->advV, f->diffV, f->dampV, f->SyA, f->SyB, f->SyD,
                          f->SyF, f->rv, f->v1, f->Vcum, f->advD_v, f->vua, f->vva,
                          f->mask_x, f->H_x, f->D_x, f->work_x, f->D_uu, f->D_uv, f->D_vu, f->D_vv, f->sync};
    for (const void* q : ptrs)
        if (!q) return GETM_ERR_ARG;
    memset(&a, 0, sizeof(a));
    a.nx = nx; a.ny = ny; a.halox = halox; a.haloy = haloy;
    a.ufirst = ufirst != 0; a.accumulate = accumulate != 0; a.friction = friction != 0;
    a.dt = timestep; a.idt = 1.0 / timestep;
    a.time = f->time;
    a.tr[0] = Transport2DArgs{f->mask_u, f->alpha_u, f->D_u, f->dpdx, f->tausx, f->corU, f->advU, f->diffU,
                              f->dampU, f->SxA, f->SxB, f->SxD, f->SxF, f->ru, f->U};
    a.tr[1] = Transport2DArgs{f->mask_v, f->alpha_v, f->D_v, f->dpdy, f->tausy, f->corV, f->advV, f->diffV,
                              f->dampV, f->SyA, f->SyB, f->SyD, f->SyF, f->rv, f->V};
    a.cor_out[0] = f->corU; a.cor_out[1] = f->corV;
    a.corf[0] = f->cor_u; a.corf[1] = f->cor_v;
    a.Ucum = f->Ucum; a.Vcum = f->Vcum;
    a.mT = f->mask_t; a.dyU = f->dy_u; a.dxV = f->dx_v; a.iareaT = f->iarea_t;
    a.z = f->z; a.zo = f->zo; a.fwf = f->fwf; a.pe = f->pe;
    a.depth = DepthArgs{nx, ny, Dmin, Dcrit, 1.0 / (Dcrit - 2 * Dmin), f->z, f->zo, f->H_t, f->H_u, f->H_v, f->H_x,
                        f->mask_t, f->mask_u, f->mask_v, f->mask_x, f->D_t, f->Dclip_t, f->work_t, f->work_u,
                        f->D_u, f->alpha_u, f->work_v, f->D_v, f->alpha_v, f->work_x, f->D_x, f->D_uu, f->D_vv,
                        f->D_uv, f->D_vu};
    a.vel = VelArgs{nx, ny, f->U, f->V, f->D_u, f->D_v, f->D_uu, f->D_uv, f->D_vu, f->D_vv, f->u1, f->v1, f->advU,
                    f->advV, f->uua, f->uva, f->vua, f->vva};
    a.fric = FricArgs{nx, ny, f->mask_u, f->mask_v, f->u1, f->v1, f->D_u, f->D_v, f->z0b_u, f->z0b_v, f->work_u,
                      f->work_v, f->ru, f->rv};
    a.spg = SpgArgs{nx, f->mask_u, f->mask_v, f->idx_u, f->idy_v, f->z, f->sp, f->H_t, f->D_t, Dmin, f->dpdx,
                    f->dpdy};
    a.taux = f->taux; a.tauy = f->tauy; a.tausx = f->tausx; a.tausy = f->tausy;
    int rc = getm_advection_2d_passes(uadv, ugrid, uugrid, uvgrid, uadv_ufirst, f->uua, f->uva, timestep, f->advD_u,
                                      f->D_uu, f->D_uv, f->advU, mixed != 0, &a.adv[0]);
    if (rc) return rc;
    rc = getm_advection_2d_passes(vadv, vgrid, vugrid, vvgrid, vadv_ufirst, f->vua, f->vva, timestep, f->advD_v,
                                  f->D_vu, f->D_vv, f->advV, mixed != 0, &a.adv[1]);
    if (rc) return rc;
    for (int d = 0; d < 2; d++)
        for (int s = 0; s < 2; s++)
            if (a.adv[d].pass[s].nx_ != nx || a.adv[d].pass[s].ny_ != ny) return GETM_ERR_ARG;
    a.Dsrc[0] = f->D_u; a.Dsrc[1] = f->D_v;
    a.advD[0] = f->advD_u; a.advD[1] = f->advD_v;
    a.advvar[0] = f->advU; a.advvar[1] = f->advV;
    a.Uo[0] = f->U; a.Uo[1] = f->V;
    a.sync = f->sync;
    return GETM_OK;
}

}  // namespace

extern "C" int getm_split2d_substep(const getm_split2d_fields* f, int nx, int ny, int halox, int haloy, int mixed,
                                    int ufirst, int accumulate, int friction, double timestep, double Dmin,
                                    double Dcrit, getm_advection* uadv, getm_grid* ugrid, getm_grid* uugrid,
                                    getm_grid* uvgrid, int uadv_ufirst, getm_advection* vadv, getm_grid* vgrid,
                                    getm_grid* vugrid, getm_grid* vvgrid, int vadv_ufirst, cudaStream_t stream)
{
    SubstepArgs a;
    int rc = substep_args(a, f, nx, ny, halox, haloy, mixed, ufirst, accumulate, friction, timestep, Dmin, Dcrit,
                          uadv, ugrid, uugrid, uvgrid, uadv_ufirst, vadv, vgrid, vugrid, vvgrid, vadv_ufirst);
    if (rc) return rc;
    return mixed ? launch_substep<true>(a, stream) : launch_substep<false>(a, stream);
}

// ---------------------------------------------------------------------------
// Substeps of many independent domains in one launch
// ---------------------------------------------------------------------------
// An ensemble of domains of uneven size (ensemble members, served requests)
// advances each member by `split` substeps per 3D step, the last of which
// runs the member's 3D step.  The other substeps of every member run here as
// one cooperative launch per substep index k: launch k advances every member
// with more than k such substeps by one substep.  The seven phases and their
// device functions are those of substep_2d_kernel; within a phase the blocks
// walk one list of block-sized work items spanning all members (512-point
// chunks, depth tiles, advection row groups or tiles), so the small planes
// of many members fill the GPU together and one set of grid barriers serves
// them all.  Members are sorted by their number of substeps (descending), so
// the members of launch k are a prefix of the table and each phase's items
// are a prefix of its offset list.  Each member keeps its own arguments, time
// step and transport order: its order at launch k of a round is its recorded
// order flipped (k + round_parity * split) times.
namespace {

constexpr int SB_PHASES = 7;

struct BatchMember {
    SubstepArgs a;
    int nsub;              // substeps without 3D step per round: takes part in launches k < nsub
    int split;             // substeps per round
    int n;                 // points nx * ny
    int pts;               // block items of a point phase
    int dtiles, dntx;      // depth tiles, and their count along x
    int adv_items[2][2];   // [U/V][pass] block items
    int adv_nbx[2][2];     // [U/V][pass] row segments (x pass) or tile columns (y pass)
};

__host__ __device__ inline int sb_div_up(int a, int b) { return (a + b - 1) / b; }

// Block items of one momentum advection pass over the plane.
template <bool MIXED>
void pass_items(const HPassArgs<double>& pa, int dir, int& items, int& nbx)
{
    if (dir == 1) {
        nbx = MIXED ? sb_div_up(pa.nx_ + 1, HX_STRIDE) : sb_div_up(pa.nx_, 32);
        items = nbx * sb_div_up(pa.ny_, SS_BY);
    } else {
        nbx = sb_div_up(pa.nx_, 32);
        const int nby = MIXED ? sb_div_up(pa.ny_ + 1, HY_STRIDE) : sb_div_up(pa.ny_, GETM_V_BY);
        items = nbx * nby;
    }
}

// Items of each phase for one member (the order within a phase is fixed
// below in batch_item).
void phase_items(const BatchMember& m, int out[SB_PHASES])
{
    out[0] = out[1] = out[2] = out[4] = m.pts;
    out[3] = m.dtiles + m.pts;
    out[5] = (m.a.friction ? m.pts : 0) + m.adv_items[0][0] + m.adv_items[1][0];
    out[6] = m.adv_items[0][1] + m.adv_items[1][1];
}

// Block item q of one pass of the momentum advection.
template <bool MIXED, typename Epi = NoEpi>
__device__ __forceinline__ void batch_pass_item(const HPassArgs<double>& pa, int dir, int nbx, int q, SubstepSmem& sm,
                                                int tx, int ty, const Epi& epi = Epi())
{
    if (dir == 1) {
        const long long row = (long long)(q / nbx) * SS_BY + ty;
        if (row < pa.ny_) {
            if constexpr (MIXED) hpass_x_inc_body<double, Epi>(pa, q % nbx, row, tx, epi);
            else hpass_x_body<double, Epi>(pa, q % nbx, row, tx, epi);
        }
    } else {
        if constexpr (MIXED) hpass_y_inc_body<double, Epi>(pa, q % nbx, q / nbx, 0, tx, ty, sm.yi, epi);
        else hpass_y_body<double, Epi>(pa, q % nbx, q / nbx, 0, tx, ty, sm.y.sQ, sm.y.sF, epi);
        __syncthreads();  // shared memory is reused by the block's next item
    }
}

// Work item q of phase ph of one member: the same operations, in the same
// order per point, as the phases of substep_2d_kernel.
template <bool MIXED>
__device__ void batch_item(const BatchMember& m, int ph, int q, int ufirst, SubstepSmem& sm, int tx, int ty)
{
    using C = typename std::conditional<MIXED, float, double>::type;
    const SubstepArgs& a = m.a;
    const int nx = a.nx, ny = a.ny;
    const int ilo = a.halox, ihi = nx - a.halox - 1, jlo = a.haloy, jhi = ny - a.haloy - 1;
    const int d1 = ufirst ? 0 : 1, d2 = 1 - d1;
    auto point = [&](int qq, int& p, int& i, int& j) {
        p = qq * SS_THREADS + ty * 32 + tx;
        j = p / nx;
        i = p - j * nx;
        return p < m.n;
    };
    auto interior = [&](int i, int j) { return i >= ilo && i <= ihi && j >= jlo && j <= jhi; };
    int p, i, j;
    switch (ph) {
    case 0:
        if (point(q, p, i, j) && interior(i, j)) transport_update<MIXED>(a.tr[d1], a.dt, p);
        break;
    case 1:
        if (point(q, p, i, j)) {
            coriolis_from<C>(a, d1, i, j);
            if (interior(i, j)) transport_update<MIXED>(a.tr[d2], a.dt, p);
        }
        break;
    case 2:
        if (point(q, p, i, j)) {
            coriolis_from<C>(a, d2, i, j);
            if (a.accumulate) accumulate_2d_point(a.tr[0].U, a.tr[1].U, a.Ucum, a.Vcum, p);
            surface_elevation_fused_point(nx, ny, a.halox, a.haloy, a.mT, a.dyU, a.dxV, a.iareaT, a.z, a.zo,
                                          a.tr[0].U, a.tr[1].U, a.fwf, a.dt, i, j);
        }
        break;
    case 3:
        if (q < m.dtiles) {
            update_depth_2d_tile<SS_BY, MIXED>(a.depth, q % m.dntx, q / m.dntx, tx, ty, sm.szh);
            __syncthreads();
        } else if (point(q - m.dtiles, p, i, j)) {
            a.fwf[p] = a.pe[p];
            if (i < nx - 1) interp_pair_point<double>(a.taux, a.tausx, p, 1, 0);
            if (j < ny - 1) interp_pair_point<double>(a.tauy, a.tausy, p, nx, 0);
        }
        break;
    case 4:
        if (point(q, p, i, j)) {
            momentum_2d_velocities_point<C>(a.vel, i, j);
            a.advD[0][p] = a.Dsrc[0][p];
            a.advD[1][p] = a.Dsrc[1][p];
            if (interior(i, j)) spg_point<MIXED>(a.spg, p);
        }
        break;
    case 5: {
        int r = q;
        if (a.friction) {
            if (r < m.pts) {
                if (point(r, p, i, j)) momentum_2d_friction_point<C>(a.fric, i, j);
                break;
            }
            r -= m.pts;
        }
        if (r < m.adv_items[0][0]) {
            batch_pass_item<MIXED>(a.adv[0].pass[0], a.adv[0].dir[0], m.adv_nbx[0][0], r, sm, tx, ty);
            break;
        }
        r -= m.adv_items[0][0];
        batch_pass_item<MIXED>(a.adv[1].pass[0], a.adv[1].dir[0], m.adv_nbx[1][0], r, sm, tx, ty);
        break;
    }
    default: {
        // the model time moves on once per member, in its first item of the
        // last phase (after the last barrier, as in substep_2d_kernel)
        if (q == 0 && tx == 0 && ty == 0 && a.time) *a.time = *a.time + a.dt;
        const int d = q < m.adv_items[0][1] ? 0 : 1;
        const int r = d == 0 ? q : q - m.adv_items[0][1];
        const ReconstructEpi epi{a.advvar[d], a.Uo[d], a.idt, jlo, jhi};
        batch_pass_item<MIXED>(a.adv[d].pass[1], a.adv[d].dir[1], m.adv_nbx[d][1], r, sm, tx, ty, epi);
        break;
    }
    }
}

// off: SB_PHASES lists of nmember + 1 item offsets (phase-major).
template <bool MIXED>
__global__ void __launch_bounds__(SS_THREADS, MIXED ? 2 : 1)
    substep_batch_kernel(const BatchMember* __restrict__ mem, const int* __restrict__ off, int nmember, int P,
                         int k, int round_parity, unsigned* sync)
{
    __shared__ SubstepSmem sm;
    __shared__ int s_ok;
    const int tx = threadIdx.x, ty = threadIdx.y;
    unsigned target = 0;
    if (tx == 0 && ty == 0) s_ok = ld_acquire(&sync[2]) == 0;
    __syncthreads();
    if (!s_ok) return;
    for (int ph = 0; ph < SB_PHASES; ph++) {
        const int* o = off + ph * (nmember + 1);
        const int total = o[P];
        for (int w = blockIdx.x; w < total; w += gridDim.x) {
            // the member of item w: the last m < P with o[m] <= w
            int lo = 0, hi = P - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (o[mid] <= w) lo = mid;
                else hi = mid - 1;
            }
            const BatchMember& m = mem[lo];
            const int ufirst = m.a.ufirst ^ ((k + round_parity * m.split) & 1);
            batch_item<MIXED>(m, ph, w - o[lo], ufirst, sm, tx, ty);
        }
        if (ph + 1 < SB_PHASES && !grid_barrier(sync, target, s_ok)) return grid_exit(sync);
    }
    grid_exit(sync);
}

template <bool MIXED>
int batch_blocks(int dev, int* blocks)
{
    static int cache[SS_MAX_DEVICES];
    static std::mutex mutex;
    if (dev < 0 || dev >= SS_MAX_DEVICES) return GETM_ERR_ARG;
    std::lock_guard<std::mutex> lock(mutex);
    if (cache[dev] == 0) {
        int sms = 0, coop = 0, per_sm = 0;
        if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
            return GETM_ERR_CUDA;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GETM_ERR_CUDA;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, substep_batch_kernel<MIXED>, SS_THREADS, 0) !=
                cudaSuccess ||
            per_sm < 1)
            return GETM_ERR_CUDA;
        cache[dev] = sms * per_sm;
    }
    *blocks = cache[dev];
    return GETM_OK;
}

}  // namespace

struct getm_substep_batch {
    int nmember, mixed;
    BatchMember* host;      // as set, in member order
    int* set;               // which members were set
    int* order;             // sorted position -> member index
    int* nsub_sorted;       // nsub of the sorted members
    BatchMember* dmem;      // device table (sorted)
    int* doff;              // device offsets
};

extern "C" int getm_substep_batch_create(int nmember, int mixed, getm_substep_batch** out)
{
    if (!out || nmember < 1) return GETM_ERR_ARG;
    getm_substep_batch* b = (getm_substep_batch*)calloc(1, sizeof(getm_substep_batch));
    if (!b) return GETM_ERR_ALLOC;
    b->nmember = nmember;
    b->mixed = mixed != 0;
    b->host = (BatchMember*)calloc(nmember, sizeof(BatchMember));
    b->set = (int*)calloc(nmember, sizeof(int));
    b->order = (int*)calloc(nmember, sizeof(int));
    b->nsub_sorted = (int*)calloc(nmember, sizeof(int));
    if (!b->host || !b->set || !b->order || !b->nsub_sorted) {
        free(b->host); free(b->set); free(b->order); free(b->nsub_sorted); free(b);
        return GETM_ERR_ALLOC;
    }
    *out = b;
    return GETM_OK;
}

extern "C" int getm_substep_batch_finalize(getm_substep_batch* b)
{
    if (!b) return GETM_OK;
    cudaFree(b->dmem);
    cudaFree(b->doff);
    free(b->host); free(b->set); free(b->order); free(b->nsub_sorted);
    free(b);
    return GETM_OK;
}

extern "C" int getm_substep_batch_set(getm_substep_batch* b, int member, int nsub, int split,
                                      const getm_split2d_fields* f, int nx, int ny, int halox, int haloy, int ufirst,
                                      int accumulate, int friction, double timestep, double Dmin, double Dcrit,
                                      getm_advection* uadv, getm_grid* ugrid, getm_grid* uugrid, getm_grid* uvgrid,
                                      int uadv_ufirst, getm_advection* vadv, getm_grid* vgrid, getm_grid* vugrid,
                                      getm_grid* vvgrid, int vadv_ufirst)
{
    if (!b || member < 0 || member >= b->nmember || nsub < 0 || split < nsub + 1 || b->dmem) return GETM_ERR_ARG;
    BatchMember& m = b->host[member];
    int rc = substep_args(m.a, f, nx, ny, halox, haloy, b->mixed, ufirst, accumulate, friction, timestep, Dmin,
                          Dcrit, uadv, ugrid, uugrid, uvgrid, uadv_ufirst, vadv, vgrid, vugrid, vvgrid, vadv_ufirst);
    if (rc) return rc;
    m.a.sync = nullptr;  // the batch launch has its own barrier words
    m.nsub = nsub;
    m.split = split;
    m.n = nx * ny;
    m.pts = sb_div_up(m.n, SS_THREADS);
    m.dntx = sb_div_up(nx + 1, UD_BX);
    m.dtiles = m.dntx * sb_div_up(ny + 1, SS_BY);
    for (int d = 0; d < 2; d++)
        for (int s = 0; s < 2; s++) {
            if (b->mixed) pass_items<true>(m.a.adv[d].pass[s], m.a.adv[d].dir[s], m.adv_items[d][s], m.adv_nbx[d][s]);
            else pass_items<false>(m.a.adv[d].pass[s], m.a.adv[d].dir[s], m.adv_items[d][s], m.adv_nbx[d][s]);
        }
    b->set[member] = 1;
    return GETM_OK;
}

extern "C" int getm_substep_batch_upload(getm_substep_batch* b)
{
    if (!b || b->dmem) return GETM_ERR_ARG;
    const int n = b->nmember;
    for (int q = 0; q < n; q++)
        if (!b->set[q]) return GETM_ERR_ARG;
    // members by their substep count, descending (stable)
    for (int q = 0; q < n; q++) b->order[q] = q;
    for (int q = 1; q < n; q++) {
        const int x = b->order[q];
        int r = q;
        while (r > 0 && b->host[b->order[r - 1]].nsub < b->host[x].nsub) {
            b->order[r] = b->order[r - 1];
            r--;
        }
        b->order[r] = x;
    }
    BatchMember* sorted = (BatchMember*)malloc(sizeof(BatchMember) * n);
    int* off = (int*)calloc((size_t)SB_PHASES * (n + 1), sizeof(int));
    if (!sorted || !off) { free(sorted); free(off); return GETM_ERR_ALLOC; }
    long long total[SB_PHASES] = {0};
    for (int q = 0; q < n; q++) {
        sorted[q] = b->host[b->order[q]];
        b->nsub_sorted[q] = sorted[q].nsub;
        int it[SB_PHASES];
        phase_items(sorted[q], it);
        for (int ph = 0; ph < SB_PHASES; ph++) {
            total[ph] += it[ph];
            off[ph * (n + 1) + q + 1] = (int)total[ph];
        }
    }
    int rc = GETM_OK;
    for (int ph = 0; ph < SB_PHASES; ph++)
        if (total[ph] >= (1ll << 31)) rc = GETM_ERR_ARG;
    if (!rc && (cudaMalloc(&b->dmem, sizeof(BatchMember) * n) != cudaSuccess ||
                cudaMalloc(&b->doff, sizeof(int) * SB_PHASES * (n + 1)) != cudaSuccess))
        rc = GETM_ERR_ALLOC;
    if (!rc && (cudaMemcpy(b->dmem, sorted, sizeof(BatchMember) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemcpy(b->doff, off, sizeof(int) * SB_PHASES * (n + 1), cudaMemcpyHostToDevice) != cudaSuccess))
        rc = GETM_ERR_CUDA;
    free(sorted);
    free(off);
    if (rc) {
        cudaFree(b->dmem); cudaFree(b->doff);
        b->dmem = nullptr; b->doff = nullptr;
    }
    return rc;
}

extern "C" int getm_substep_batch_participants(const getm_substep_batch* b, int k, int* count)
{
    if (!b || !count || k < 0) return GETM_ERR_ARG;
    int P = 0;
    while (P < b->nmember && b->nsub_sorted[P] > k) P++;
    *count = P;
    return GETM_OK;
}

extern "C" int getm_substep_batch_launch(getm_substep_batch* b, int k, int round_parity, unsigned int* sync,
                                         cudaStream_t stream)
{
    if (!b || !b->dmem || !sync || k < 0 || round_parity < 0 || round_parity > 1) return GETM_ERR_ARG;
    int P = 0;
    getm_substep_batch_participants(b, k, &P);
    if (P == 0) return GETM_OK;
    int dev = 0, blocks = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GETM_ERR_CUDA;
    int rc = b->mixed ? batch_blocks<true>(dev, &blocks) : batch_blocks<false>(dev, &blocks);
    if (rc) return rc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(32, SS_BY);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const BatchMember* mem = b->dmem;
    const int* off = b->doff;
    const int n = b->nmember;
    cudaError_t e = b->mixed ? cudaLaunchKernelEx(&cfg, substep_batch_kernel<true>, mem, off, n, P, k, round_parity, sync)
                             : cudaLaunchKernelEx(&cfg, substep_batch_kernel<false>, mem, off, n, P, k, round_parity,
                                                  sync);
    if (e != cudaSuccess) return GETM_ERR_CUDA;
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}
