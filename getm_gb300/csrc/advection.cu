// TVD directional-split advection (pygetm.operators.Advection) for sm_103a.
//
// Reference: src/operators/advection_schemes/advection.F90.template (u2d :23-121,
// v2d :123-221, w3d :223-374), limiters.h, python/src/wrapper.F90:188-273 and
// the split sequencing of python/pygetm/operators.py:52-193.
//
// GB300 design
// * Horizontal passes are one kernel per direction and stage, batched over all
//   tracers: the face geometry (mask, transport QU, Courant number, upwind
//   side) and the layer-thickness update are computed once per cell and
//   reused for every tracer.  Memory traffic per pass is the algorithmic
//   minimum: read u, hu, h, var; write h, var.
// * The reference updates var and h in place after computing all face fluxes
//   of a layer.  A GPU block cannot see its neighbours' updates in order, so
//   each pass reads from one buffer and writes a complete copy to another
//   (ping-pong through handle-owned work buffers); the stage sequence is laid
//   out so the final stage lands in the caller's arrays.
// * x-direction: a warp covers 32 consecutive cells of a row; each lane
//   computes the flux through its east face and receives the west face from
//   its neighbour with a shuffle (lane 0 computes one extra face).
// * y-direction: a 32 x BY block; each thread computes its north face and the
//   south face comes from shared memory (row 0 computes one extra face).
// * Vertical pass: one thread per water column, sweeping k with a register
//   window (the per-column update is in place, as in the reference).  The
//   adaptive sub-stepping (itersmax = 200, restart semantics of
//   template :286-368) runs through handle-owned column work arrays.
#include <stdlib.h>
#include <string.h>

#include <cuda_pipeline.h>

#include "advection_passes.cuh"


// ---------------------------------------------------------------------------
// grid handles
// ---------------------------------------------------------------------------
extern "C" int getm_create_grid(int imin, int imax, int jmin, int jmax, int kmin, int kmax,
                                int halox, int haloy, getm_grid** grid)
{
    if (!grid || imax < imin || jmax < jmin || kmax < kmin - 1 || halox < 0 || haloy < 0)
        return GETM_ERR_ARG;
    getm_grid* g = (getm_grid*)calloc(1, sizeof(getm_grid));
    if (!g) return GETM_ERR_ALLOC;
    g->imin = imin; g->imax = imax; g->jmin = jmin; g->jmax = jmax;
    g->kmin = kmin; g->kmax = kmax; g->halox = halox; g->haloy = haloy;
    g->nx_ = imax - imin + 1 + 2 * halox;
    g->ny_ = jmax - jmin + 1 + 2 * haloy;
    *grid = g;
    return GETM_OK;
}

extern "C" int getm_grid_finalize(getm_grid* grid)
{
    if (grid) {
        cudaFree(grid->dx_f); cudaFree(grid->dy_f); cudaFree(grid->idx_f);
        cudaFree(grid->idy_f); cudaFree(grid->iarea_f);
    }
    free(grid);
    return GETM_OK;
}

__global__ void to_float_kernel(long long n, const double* src, float* dst)
{
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) dst[p] = (float)src[p];
}

// The float copies of a grid's metrics, converted on `stream` after every
// earlier write of the metrics on that stream, and complete on return (the
// wait is for `stream` only).
static int grid_float_metrics_on(getm_grid* g, cudaStream_t stream)
{
    const long long n = (long long)g->nx_ * g->ny_;
    const double* src[5] = {g->dx, g->dy, g->idx, g->idy, g->iarea};
    float** dst[5] = {&g->dx_f, &g->dy_f, &g->idx_f, &g->idy_f, &g->iarea_f};
    for (int q = 0; q < 5; q++) {
        if (!src[q]) continue;  // metric not registered on this grid
        float* d = NULL;
        if (cudaMalloc(&d, n * sizeof(float)) != cudaSuccess) return GETM_ERR_ALLOC;
        to_float_kernel<<<getm_div_up(n, 256), 256, 0, stream>>>(n, src[q], d);
        GETM_CHECK_LAUNCH();
        *dst[q] = d;
    }
    if (!g->iarea_f) {  // grids without cell areas (velocity grids): mark as built
        if (cudaMalloc(&g->iarea_f, sizeof(float)) != cudaSuccess) return GETM_ERR_ALLOC;
    }
    if (cudaStreamSynchronize(stream) != cudaSuccess) return GETM_ERR_CUDA;
    return GETM_OK;
}

// First use by a float kernel of a grid whose copies were not made with
// getm_grid_float_metrics: the metrics may have been written on any stream,
// so the conversion is ordered after all work on the device.
int getm_grid_f32_metrics(getm_grid* g, cudaStream_t stream)
{
    if (!g) return GETM_ERR_ARG;
    if (g->iarea_f) return GETM_OK;  // built last: its presence means all are there
    if (cudaDeviceSynchronize() != cudaSuccess) return GETM_ERR_CUDA;
    return grid_float_metrics_on(g, stream);
}

extern "C" int getm_grid_float_metrics(getm_grid* g, cudaStream_t stream)
{
    if (!g) return GETM_ERR_ARG;
    if (g->iarea_f) return GETM_OK;
    return grid_float_metrics_on(g, stream);
}

extern "C" int getm_grid_set_array(getm_grid* g, const char* name, void* p)
{
    if (!g || !name) return GETM_ERR_ARG;
    if (!strcmp(name, "mask")) g->mask = (const int*)p;
    else if (!strcmp(name, "dx")) g->dx = (const double*)p;
    else if (!strcmp(name, "dy")) g->dy = (const double*)p;
    else if (!strcmp(name, "idx")) g->idx = (const double*)p;
    else if (!strcmp(name, "idy")) g->idy = (const double*)p;
    else if (!strcmp(name, "iarea")) g->iarea = (const double*)p;
    else if (!strcmp(name, "area")) g->area = (const double*)p;
    else return GETM_ERR_ARG;
    return GETM_OK;
}

// ---------------------------------------------------------------------------
// advection handle: scheme plus device work buffers (grown on demand)
// ---------------------------------------------------------------------------
struct getm_advection {
    int scheme;
    getm_grid* tgrid;
    size_t n3;                 // elements of one 3D field the buffers are sized for
    double* hbuf[2];           // layer-thickness ping-pong buffers
    double* colbuf[2];         // vertical sub-stepping work arrays (haux: n3, faux: 2 n3 doubles)
    double* tmp[GETM_MAX_BATCH * 8];  // per-tracer ping-pong buffers
    int ntmp;
    int* status;               // device status word (GETM_ERR_ITERS)
};

static void adv_free_buffers(getm_advection* a)
{
    // (cudaFree waits for the whole device: never called without a buffer)
    for (int i = 0; i < 2; i++) if (a->hbuf[i]) { cudaFree(a->hbuf[i]); a->hbuf[i] = NULL; }
    for (int i = 0; i < 2; i++) if (a->colbuf[i]) { cudaFree(a->colbuf[i]); a->colbuf[i] = NULL; }
    for (int i = 0; i < a->ntmp; i++) if (a->tmp[i]) { cudaFree(a->tmp[i]); a->tmp[i] = NULL; }
    a->ntmp = 0;
    a->n3 = 0;
}

// Make sure the work buffers can hold 3D fields of n3 elements and ntracer
// per-tracer ping-pong copies.  Allocation happens on first use only (so a
// warm-up call before stream capture makes later calls capturable).
static int adv_reserve(getm_advection* a, size_t n3, int ntracer)
{
    if (ntracer > GETM_MAX_BATCH * 8) return GETM_ERR_ARG;
    if (n3 > a->n3) {
        adv_free_buffers(a);
        for (int i = 0; i < 2; i++)
            if (cudaMalloc(&a->hbuf[i], n3 * sizeof(double)) != cudaSuccess) return GETM_ERR_ALLOC;
        // colbuf[1] holds the intermediate sub-steps of a pair of fields
        // stepped together by the w pass (two fields of up to 8 bytes)
        if (cudaMalloc(&a->colbuf[0], n3 * sizeof(double)) != cudaSuccess) return GETM_ERR_ALLOC;
        if (cudaMalloc(&a->colbuf[1], 2 * n3 * sizeof(double)) != cudaSuccess) return GETM_ERR_ALLOC;
        a->n3 = n3;
    }
    while (a->ntmp < ntracer) {
        if (cudaMalloc(&a->tmp[a->ntmp], a->n3 * sizeof(double)) != cudaSuccess) return GETM_ERR_ALLOC;
        a->ntmp++;
    }
    return GETM_OK;
}

extern "C" int getm_advection_create(int scheme, getm_grid* tgrid, getm_advection** out)
{
    if (!out || scheme < GETM_SCHEME_HSIMT || scheme > GETM_SCHEME_UPSTREAM) return GETM_ERR_ARG;
    getm_advection* a = (getm_advection*)calloc(1, sizeof(getm_advection));
    if (!a) return GETM_ERR_ALLOC;
    a->scheme = scheme;
    a->tgrid = tgrid;
    if (cudaMalloc(&a->status, sizeof(int)) != cudaSuccess) { free(a); return GETM_ERR_ALLOC; }
    cudaMemset(a->status, 0, sizeof(int));
    *out = a;
    return GETM_OK;
}

extern "C" int getm_advection_finalize(getm_advection* a)
{
    if (!a) return GETM_OK;
    adv_free_buffers(a);
    cudaFree(a->status);
    free(a);
    return GETM_OK;
}

extern "C" int getm_advection_get_status(getm_advection* a, cudaStream_t stream)
{
    if (!a) return GETM_ERR_ARG;
    int h = 0;
    if (cudaMemcpyAsync(&h, a->status, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess) return GETM_ERR_CUDA;
    if (cudaStreamSynchronize(stream) != cudaSuccess) return GETM_ERR_CUDA;
    return h;
}

// ---- kernels (one pass per launch) ------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) hpass_x_kernel(HPassArgs<T> a)
{
    hpass_x_body<T>(a, blockIdx.x, (long long)blockIdx.y * blockDim.y + threadIdx.y, threadIdx.x);
}

template <typename T>
__global__ void __launch_bounds__(32 * GETM_V_BY) hpass_y_kernel(HPassArgs<T> a)
{
    __shared__ double sQ[GETM_V_BY][32];
    __shared__ T sF[GETM_V_BY][32];
    hpass_y_body<T>(a, blockIdx.x, blockIdx.y, blockIdx.z, threadIdx.x, threadIdx.y, sQ, sF);
}

// grid (segments, ceil(ny_ / 8), nk): warp (ty) of block (x, y, k) owns row j = 8 y + ty of layer k
template <typename S, typename V = S>
__global__ void __launch_bounds__(256) hpass_x_inc_kernel(HPassArgs<S, V> a)
{
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= a.ny_) return;  // whole warp
    hpass_x_inc_rows<S, 1, NoEpi, V>(a, blockIdx.x, j, blockIdx.z, threadIdx.x);
}

// grid (1, ceil(ny_ / rows), nk): warp (ty) of block (0, y, k) sweeps row j = rows y + ty of layer k
template <typename S, typename V = S>
__global__ void __launch_bounds__(256) hpass_x_vec_kernel(HPassArgs<S, V> a)
{
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= a.ny_) return;  // whole warp
    hpass_x_vec_row<S, V>(a, j, blockIdx.z, threadIdx.x);
}

// The four-cells-per-lane x pass applies: rows of whole 16-byte vectors and
// every pointer it reads or writes 16-byte aligned.
template <typename S, typename V>
static bool xpass_vec_ok(const HPassArgs<S, V>& a)
{
    if (a.nk < 2 || a.nx_ % 4 != 0 || a.ntracer > GETM_MAX_BATCH) return false;
    auto al = [](const void* p) { return ((uintptr_t)p & 15u) == 0; };
    if (!al(a.umask) || !al(a.tmask) || !al(a.dy_f) || !al(a.idx_f) || !al(a.iA_f) || !al(a.u) || !al(a.hu) ||
        !al(a.h_in) || !al(a.h_out) || (a.Ah && !al(a.Ah)))
        return false;
    for (int t = 0; t < a.ntracer; t++)
        if (!al(a.fin[t]) || !al(a.fout[t])) return false;
    return true;
}

template <typename S, typename V = S>
__global__ void __launch_bounds__(32 * HY_BY) hpass_y_inc_kernel(HPassArgs<S, V> a)
{
    __shared__ YIncSmem<S> sm;
    hpass_y_inc_body<S, NoEpi, V>(a, blockIdx.x, blockIdx.y, blockIdx.z, threadIdx.x, threadIdx.y, sm);
}

template <typename S, int NT, typename V = S>
__global__ void __launch_bounds__(256) hpass_y_march_kernel(HPassArgs<S, V> a, int nchunk)
{
    const int w = blockIdx.y * blockDim.y + threadIdx.y;
    const int chunk = w % nchunk, k = w / nchunk;
    if (k >= a.nk) return;  // whole warp
    // one sweep per group of NT tracers; with no tracers one sweep updates h
    for (int t0 = 0; t0 == 0 || t0 < a.ntracer; t0 += NT)
        hpass_y_march_body<S, NT, V>(a, blockIdx.x, chunk, k, threadIdx.x, t0);
}

// Launch one horizontal pass in increment form (any storage type S,
// velocity type V).
template <typename S, typename V = S>
static int launch_hpass_inc(int direction, HPassArgs<S, V>& a, cudaStream_t stream)
{
    if (direction == 1) {
        const int rows = getm_tune(GETM_TUNE_XPASS_ROWS);
        dim3 block(32, rows);
        if (getm_tune(GETM_TUNE_XPASS_VEC) && xpass_vec_ok(a)) {
            dim3 grid(1, getm_div_up(a.ny_, rows), a.nk);
            hpass_x_vec_kernel<S, V><<<grid, block, 0, stream>>>(a);
        } else {
            // lane 0 of the first segment handles the face west of cell 0
            dim3 grid(getm_div_up(a.nx_ + 1, HX_STRIDE), getm_div_up(a.ny_, rows), a.nk);
            hpass_x_inc_kernel<S, V><<<grid, block, 0, stream>>>(a);
        }
    } else if (a.nk < 4) {
        // a single plane: too few columns x layers for marching warps to fill
        // the GPU, so blocks of 32 x HY_BY threads cover tiles instead
        dim3 block(32, HY_BY);
        dim3 grid(getm_div_up(a.nx_, 32), getm_div_up(a.ny_ + 1, HY_STRIDE), a.nk);
        hpass_y_inc_kernel<S, V><<<grid, block, 0, stream>>>(a);
    } else {
        a.ych = getm_tune(GETM_TUNE_YMARCH_CHUNK);
        const int nchunk = getm_div_up(a.ny_, a.ych);
        dim3 block(32, 8);
        dim3 grid(getm_div_up(a.nx_, 32), getm_div_up((long long)nchunk * a.nk, 8));
        if (a.ntracer >= 2) hpass_y_march_kernel<S, 2, V><<<grid, block, 0, stream>>>(a, nchunk);
        else hpass_y_march_kernel<S, 1, V><<<grid, block, 0, stream>>>(a, nchunk);
    }
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

template <typename T, typename V = T>
static int launch_hpass(int direction, HPassArgs<T, V>& a, cudaStream_t stream)
{
    if constexpr (getm_increment_form<T> || !std::is_same<T, V>::value) {
        return launch_hpass_inc<T, V>(direction, a, stream);
    } else {
        if (a.increment) return launch_hpass_inc<T, V>(direction, a, stream);
        if (direction == 1) {
            const int BY = 8;
            dim3 block(32, BY);
            dim3 grid(getm_div_up(a.nx_, 32), getm_div_up((long long)a.ny_ * a.nk, BY));
            hpass_x_kernel<T><<<grid, block, 0, stream>>>(a);
        } else {
            dim3 block(32, GETM_V_BY);
            dim3 grid(getm_div_up(a.nx_, 32), getm_div_up(a.ny_, GETM_V_BY), a.nk);
            hpass_y_kernel<T><<<grid, block, 0, stream>>>(a);
        }
        GETM_CHECK_LAUNCH();
        return GETM_OK;
    }
}

// Fill the direction-dependent fields of HPassArgs from the grid handles
// (wrapper.F90:240-253: direction 1 passes ugrid mask/idx/dy, 2 passes vgrid
// mask/dx/idy).
template <typename T, typename V = T>
static int hpass_setup(HPassArgs<T, V>& a, int direction, const getm_advection* adv, const getm_grid* tg,
                       const getm_grid* vg, int nk, const V* u, const double* Ah, double dt, const double* hu,
                       int increment = 0)
{
    if (!tg || !vg || !u || !hu) return GETM_ERR_ARG;
    if (tg->halox < 2 || tg->haloy < 2) return GETM_ERR_ARG;
    if (!tg->mask || !tg->iarea || !vg->mask) return GETM_ERR_ARG;
    memset(&a, 0, sizeof(a));
    a.nx_ = tg->nx_; a.ny_ = tg->ny_; a.nk = nk;
    a.plane = (long long)tg->nx_ * tg->ny_;
    a.ilo = tg->halox; a.ihi = tg->halox + (tg->imax - tg->imin);
    a.jlo = tg->haloy; a.jhi = tg->haloy + (tg->jmax - tg->jmin);
    a.umask = vg->mask;
    if (direction == 1) { a.idx = vg->idx; a.dy = vg->dy; }
    else { a.idx = vg->idy; a.dy = vg->dx; }
    if (!a.idx || !a.dy) return GETM_ERR_ARG;
    a.tmask = tg->mask; a.iA = tg->iarea; a.Ah = Ah; a.u = u; a.hu = hu; a.dt = dt;
    a.scheme = adv->scheme;
    a.dtf = (float)dt;
    if (getm_increment_form<T> || !std::is_same<T, V>::value || increment) {
        a.increment = 1;
        int rc = getm_grid_f32_metrics(const_cast<getm_grid*>(tg), 0);
        if (!rc) rc = getm_grid_f32_metrics(const_cast<getm_grid*>(vg), 0);
        if (rc) return rc;
        a.iA_f = tg->iarea_f;
        if (direction == 1) { a.idx_f = vg->idx_f; a.dy_f = vg->dy_f; }
        else { a.idx_f = vg->idy_f; a.dy_f = vg->dx_f; }
        if (!a.iA_f || !a.idx_f || !a.dy_f) return GETM_ERR_ARG;
    }
    return GETM_OK;
}

// Run one horizontal stage for ntracer tracers, chunked by GETM_MAX_BATCH.
template <typename T, typename V = T>
static int run_hstage(HPassArgs<T, V>& a, int direction, const double* h_in, double* h_out, int ntracer,
                      const T* const* fin, T* const* fout, cudaStream_t stream)
{
    a.h_in = h_in; a.h_out = h_out;
    int done = 0;
    do {
        int n = ntracer - done;
        if (n > GETM_MAX_BATCH) n = GETM_MAX_BATCH;
        a.ntracer = n;
        for (int t = 0; t < n; t++) { a.fin[t] = fin[done + t]; a.fout[t] = fout[done + t]; }
        int rc = launch_hpass<T, V>(direction, a, stream);
        if (rc) return rc;
        done += n;
    } while (done < ntracer);
    return GETM_OK;
}

// ---------------------------------------------------------------------------
// vertical pass (template w3d :223-374)
// ---------------------------------------------------------------------------
// T: the advected fields; V: w and w_var (T unless given).  T = double, V =
// float is the mixed form with FP64 tracer storage (increment form).
template <typename T, typename V = T>
struct WPassArgs {
    int nx_, ny_, nz;
    long long plane;
    int ilo, ihi, jlo, jhi;
    const int* tmask;
    const V* w;                 // nz+1 levels
    const double* h_in;         // layer thickness at stage start (not modified)
    double* h_out;              // layer thickness after the pass (last tracer's)
    double* haux;               // column work arrays for sub-stepping (nz levels)
    T* faux;
    double dt;
    int scheme;
    int ntracer;
    int* status;
    const V* wvar[GETM_MAX_BATCH];
    T* f[GETM_MAX_BATCH];       // updated in place
};

// One sub-step over a column: reads (hs, fs) levels 0..nz-1 (C), writes
// (hd, fdst).  hs == hd / fs == fdst (in place) is allowed: every level is
// read into the register window before it is overwritten.  The Courant number
// |w_var| dt / min(h) * itersm1 equals cfls(k)*itersm1 of the reference
// (cfls = |w_var| dt / min(haux), haux = the sub-step's start thickness).
template <typename T>
__device__ void w_substep(const WPassArgs<T>& a, long long c, const T* wv, const double* hs, const T* fs,
                          double* hd, T* fdst, double dtk, double itersm1)
{
    const long long P = a.plane;
    const int nz = a.nz;
    T fkm1 = T(0), fk = fs[c], fk1 = (nz > 1) ? fs[c + P] : T(0);
    double hk = hs[c], hk1 = (nz > 1) ? hs[c + P] : 0.0;
    T fluxm = T(0);  // flux(k-1), flux(0) = 0
    T wkm1 = a.w[c];
    for (int k = 0; k < nz; k++) {
        // flux through the interface above C level k (Fortran interface k+1)
        T flux = T(0);
        T fk2 = T(0);
        double hk2 = 0.0;
        if (k + 2 < nz) { fk2 = fs[c + (k + 2) * P]; hk2 = hs[c + (k + 2) * P]; }
        if (k < nz - 1) {
            T wvk = wv[c + (k + 1) * P];
            T cfl = fabs(wvk) * (T)a.dt / (T)fmin(hk, hk1) * (T)itersm1;
            T fu, fuu, fdn;
            if (wvk > T(0)) {
                fu = fk;
                fuu = (k > 0) ? fkm1 : fu;
                fdn = fk1;
            } else {
                fu = fk1;
                fuu = (k < nz - 2) ? fk2 : fu;
                fdn = fk;
            }
            fu = getm_tvd_face<T>(a.scheme, fuu, fu, fdn, cfl);
            flux = wvk * fu;
        }
        T wk = a.w[c + (k + 1) * P];
        double dh = dtk * ((double)wk - (double)wkm1);
        double hn = hk - dh;
        T advn = flux - fluxm;
        hd[c + k * P] = hn;
        T hfo = (T)hk * fk;
        fdst[c + k * P] = (hfo - (T)dtk * advn) / (T)hn;
        // shift window
        fluxm = flux; wkm1 = wk;
        fkm1 = fk; fk = fk1; fk1 = fk2;
        hk = hk1; hk1 = hk2;
    }
}

// Mixed form of w_substep: the increment form of the horizontal passes in
// the vertical (see hpass_x_inc_kernel).  With flux_k = W_k f + e_k at the
// interface above level k (W_k = w_var there, 0 at the surface) and
// dh = dtk (w_k - w_{k-1}), the reference update equals
//     f + dtk ((w_k - W_k - w_{k-1} + W_{k-1}) f - e_k + e'_{k-1}) / hn
// with e_k = W_k (face_k - f_k) and e'_{k-1} = W_{k-1} (face_{k-1} - f_k).
// NT fields advected with the same w_var share every thickness and velocity
// load and the face constants; each field keeps its own window.
// The operands of the levels a column sweep will need are staged W_STAGE
// levels ahead into a per-thread ring in shared memory by asynchronous
// copies (cp.async): the loads of W_STAGE levels are in flight without
// holding registers, where register prefetch reached two levels.  Each
// thread reads back only the slots it filled, so no block barrier is
// involved; a slot is refilled only after its level was read.
constexpr int W_STAGE = 6;
constexpr int W_RING = W_STAGE + 1;

template <typename S>
struct WRing {
    double* h;  // h of level L at h[(L % W_RING) * 32]
    S* f;       // field q of level L at f[((L % W_RING) * 2 + q) * 32]
    float* W;   // the field's vertical velocity (w_var) of level L
    float* w;   // w of level L (nz + 1 interfaces)
};

template <typename S>
constexpr size_t w_ring_bytes_per_thread()
{
    return (size_t)W_RING * (sizeof(double) + 2 * sizeof(S) + 2 * sizeof(float));
}

// the ring of thread (lane, warp) in the block's dynamic shared memory
// (doubles first, so every slot is naturally aligned)
template <typename S>
__device__ __forceinline__ WRing<S> w_ring(unsigned char* smem, int nwarps, int warp, int lane)
{
    WRing<S> r;
    double* hb = reinterpret_cast<double*>(smem);
    S* fb = reinterpret_cast<S*>(hb + (size_t)nwarps * W_RING * 32);
    float* Wb = reinterpret_cast<float*>(fb + (size_t)nwarps * W_RING * 64);
    float* wb = Wb + (size_t)nwarps * W_RING * 32;
    r.h = hb + (size_t)warp * W_RING * 32 + lane;
    r.f = fb + (size_t)warp * W_RING * 64 + lane;
    r.W = Wb + (size_t)warp * W_RING * 32 + lane;
    r.w = wb + (size_t)warp * W_RING * 32 + lane;
    return r;
}

template <int NT, typename S>
__device__ void w_substep_inc(const WPassArgs<S, float>& a, long long c, const float* wv, const double* hs,
                              const S* const (&fs)[NT], double* hd, S* const (&fdst)[NT], double dtk,
                              double itersm1, const WRing<S>& ring)
{
    const long long P = a.plane;
    const int nz = a.nz;
    const float dtkf = (float)dtk, itf = (float)itersm1, dtf = (float)a.dt;
    S fk[NT], fk1[NT];
    float erm[NT];  // erm: e'_{k-1}, interface below, deviation from level k
    // the differences f[k+1] - f[k] (dk) and f[k] - f[k-1] (dkm1), narrowed:
    // each is formed once, as the level above's is needed next (the
    // downwind-side difference f[k+1] - f[k+2] is -(f[k+2] - f[k+1]), the
    // same bits up to the sign of a zero, which the limiter ignores)
    float dk[NT], dkm1[NT];
#pragma unroll
    for (int q = 0; q < NT; q++) {
        fk[q] = fs[q][c];
        fk1[q] = (nz > 1) ? fs[q][c + P] : S(0);
        dk[q] = (nz > 1) ? inc_f<S>(fk1[q] - fk[q]) : 0.f;
        dkm1[q] = 0.f;
        erm[q] = 0.f;
    }
    double hk = hs[c], hk1 = (nz > 1) ? hs[c + P] : 0.0;
    float hkf = getm_d2f_approx(hk), hk1f = getm_d2f_approx(hk1);
    float Wm = 0.f;    // W_{k-1} (0 below the bottom level)
    float wkm1 = a.w[c];
    // the interface values above level k, one level ahead
    float Wn = (nz > 1) ? wv[c + P] : 0.f;
    float wkn = a.w[c + P];
    // level L's operands into its slot (nothing past the column), one
    // commit group per level
    auto stage = [&](int L) {
        const int s = L % W_RING;
        if (L < nz) {
#pragma unroll
            for (int q = 0; q < NT; q++)
                __pipeline_memcpy_async(&ring.f[(s * 2 + q) * 32], &fs[q][c + (long long)L * P], sizeof(S));
            __pipeline_memcpy_async(&ring.h[s * 32], &hs[c + (long long)L * P], sizeof(double));
            __pipeline_memcpy_async(&ring.W[s * 32], &wv[c + (long long)L * P], sizeof(float));
        }
        if (L <= nz) __pipeline_memcpy_async(&ring.w[s * 32], &a.w[c + (long long)L * P], sizeof(float));
        __pipeline_commit();
    };
    for (int L = 2; L < 2 + W_STAGE; L++) stage(L);
    for (int k = 0; k < nz; k++) {
        // level k + 2: its group is the oldest of the W_STAGE in flight
        __pipeline_wait_prior(W_STAGE - 1);
        const int s2 = (k + 2) % W_RING;
        S fk2[NT];
        double hk2 = 0.0;
#pragma unroll
        for (int q = 0; q < NT; q++) fk2[q] = (k + 2 < nz) ? ring.f[(s2 * 2 + q) * 32] : S(0);
        if (k + 2 < nz) hk2 = ring.h[s2 * 32];
        const float W = Wn;
        const float wk = wkn;
        Wn = (k + 1 < nz - 1) ? ring.W[s2 * 32] : 0.f;
        wkn = (k + 1 < nz) ? ring.w[s2 * 32] : 0.f;
        stage(k + 2 + W_STAGE);  // into the slot of level k + 1, read at k - 1
        const float cfl = fabsf(W) * dtf / fminf(hkf, hk1f) * itf;
        const TvdFaceF tf = getm_tvd_face_f(a.scheme, cfl);
        const float dh = dtkf * (wk - wkm1);
        const double hn = hk - getm_f2d(dh);
        hd[c + k * P] = hn;
#pragma unroll
        for (int q = 0; q < NT; q++) {
            // differences of neighbouring values in the storage type, then
            // narrowed (exact for float storage)
            const float dn = (k + 2 < nz) ? inc_f<S>(fk2[q] - fk1[q]) : 0.f;
            float el = 0.f, er = 0.f;
            if (k < nz - 1) {
                const float d = dk[q];
                float dev;
                if (W > 0.f) dev = getm_tvd_dev_f(tf, d, dkm1[q]);
                else dev = getm_tvd_dev_f(tf, -d, -dn);
                el = W * (W > 0.f ? dev : d + dev);
                er = W * (W > 0.f ? dev - d : dev);
            }
            fdst[q][c + k * P] =
                inc_add<S>(fk[q], dtkf * (((wk - W) - (wkm1 - Wm)) * inc_f<S>(fk[q]) - el + erm[q]) / (hkf - dh));
            erm[q] = er;
            dkm1[q] = dk[q]; dk[q] = dn;
            fk[q] = fk1[q]; fk1[q] = fk2[q];
        }
        Wm = W; wkm1 = wk;
        hk = hk1; hk1 = hk2;
        hkf = hk1f; hk1f = getm_d2f_approx(hk2);
    }
    __pipeline_wait_prior(0);  // the ring is free for the next sweep
}

// Largest Courant number over the interior interfaces of a column
// (template :274, :294, :300).  Returns -1 when nz == 1 (no interfaces).
template <typename T, typename V>
__device__ double w_maxcfl(const WPassArgs<T, V>& a, long long c, const V* wv, const double* hs)
{
    const long long P = a.plane;
    V cmax = V(-1);
    if constexpr (getm_increment_form<V>) {
        const float dtf = (float)a.dt;
        float hk = getm_d2f_approx(hs[c]);
        for (int k = 1; k < a.nz; k++) {
            const float hk1 = getm_d2f_approx(hs[c + k * P]);
            const float cfl = fabsf(wv[c + k * P]) * dtf / fminf(hk, hk1);
            if (k == 1 || cfl > cmax) cmax = cfl;
            hk = hk1;
        }
        return (double)cmax;
    }
    double hk = hs[c];
    for (int k = 1; k < a.nz; k++) {
        double hk1 = hs[c + k * P];
        V cfl = fabs(wv[c + k * P]) * (V)a.dt / (V)fmin(hk, hk1);
        if (k == 1 || cfl > cmax) cmax = cfl;
        hk = hk1;
    }
    return (double)cmax;
}

__device__ __forceinline__ int w_iters_from(double cfl)
{
    if (!(cfl > 1.0)) return 1;               // includes nz == 1 and NaN
    double c = ceil(cfl);
    return c > 1e9 ? 1000000000 : (int)c;
}

// Thread per column.
// T: fields; V: velocities.  Blocks of 32 columns by GETM_TUNE_COLUMN_ROWS
// rows (row lengths need not be multiples of 128 columns).
template <typename T, typename V = T>
__global__ void __launch_bounds__(128, getm_increment_form<V> ? 7 : 1) wpass_kernel(WPassArgs<T, V> a)
{
    extern __shared__ __align__(16) unsigned char w_smem[];
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= a.nx_ || j >= a.ny_) return;
    const long long c = (long long)j * a.nx_ + i;
    const bool touched = i >= a.ilo && i <= a.ihi && j >= a.jlo && j <= a.jhi && a.tmask[c] == 1 && a.ntracer > 0;
    if (!touched) {
        // a column the pass does not update keeps its thickness (h_out must
        // be a complete field: it is a ping-pong buffer)
        if (a.h_out != a.h_in)
            for (int k = 0; k < a.nz; k++) a.h_out[c + k * a.plane] = a.h_in[c + k * a.plane];
        return;
    }
    const int itersmax = 200;
    // mixed form: two consecutive fields with the same w_var are stepped
    // together (the sub-step count depends only on w_var and h)
    constexpr bool inc = getm_increment_form<V>;
    // the second field's intermediate sub-steps use the upper half of the
    // column work array colbuf[1] (2 n3 doubles)
    constexpr bool pairs = inc;
    for (int t = 0; t < a.ntracer;) {
        const int nt = (pairs && t + 1 < a.ntracer && a.wvar[t + 1] == a.wvar[t]) ? 2 : 1;
        const V* wv = a.wvar[t];
        T* f = a.f[t];
        int iters = 1;
        double itersm1 = 1.0, dtk = a.dt;
        int it = 1;
        while (it <= iters) {
            const double* hs = (it == 1) ? a.h_in : a.haux;
            const T* fs = (it == 1) ? f : a.faux;
            if (iters < itersmax) {
                int iters_new = w_iters_from(w_maxcfl(a, c, wv, hs));
                if (iters_new > iters) {
                    if (iters_new > itersmax) {
                        iters = itersmax;
                        atomicOr(a.status, 1 << GETM_ERR_ITERS);
                    } else {
                        iters = iters_new;
                    }
                    itersm1 = 1.0 / iters;
                    dtk = a.dt * itersm1;
                    if (it > 1) { it = 1; continue; }
                }
            }
            // The last sub-step writes the tracer in place and the thickness
            // into haux (the stage's h_in must survive for the next tracer);
            // the last tracer's last sub-step writes the thickness straight
            // into h_out, the pass's result.
            T* fd = (it == iters) ? f : a.faux;
            double* hd = (it == iters && t + nt == a.ntracer) ? a.h_out : a.haux;
            if constexpr (inc) {
                if (pairs && nt == 2) {
                    T* f2 = a.f[t + 1];
                    T* faux2 = a.faux + a.plane * a.nz;
                    const T* const fs2[2] = {fs, (it == 1) ? f2 : faux2};
                    T* const fd2[2] = {fd, (it == iters) ? f2 : faux2};
                    w_substep_inc<2, T>(a, c, wv, hs, fs2, hd, fd2, dtk, itersm1,
                                        w_ring<T>(w_smem, blockDim.y, threadIdx.y, threadIdx.x));
                } else {
                    const T* const fs1[1] = {fs};
                    T* const fd1[1] = {fd};
                    w_substep_inc<1, T>(a, c, wv, hs, fs1, hd, fd1, dtk, itersm1,
                                        w_ring<T>(w_smem, blockDim.y, threadIdx.y, threadIdx.x));
                }
            } else {
                w_substep(a, c, wv, hs, fs, hd, fd, dtk, itersm1);
            }
            it++;
        }
        t += nt;
    }
}

template <typename T, typename V = T>
static int run_wstage(getm_advection* adv, const getm_grid* tg, const V* w, const V* const* wvar, double dt,
                      const double* h_in, double* h_out, int ntracer, T* const* f, cudaStream_t stream)
{
    WPassArgs<T, V> a;
    memset(&a, 0, sizeof(a));
    a.nx_ = tg->nx_; a.ny_ = tg->ny_; a.nz = tg->kmax - tg->kmin + 1;
    a.plane = (long long)tg->nx_ * tg->ny_;
    a.ilo = tg->halox; a.ihi = tg->halox + (tg->imax - tg->imin);
    a.jlo = tg->haloy; a.jhi = tg->haloy + (tg->jmax - tg->jmin);
    a.tmask = tg->mask; a.w = w; a.dt = dt; a.scheme = adv->scheme; a.status = adv->status;
    a.haux = adv->colbuf[0]; a.faux = (T*)adv->colbuf[1];
    if (a.nz < 1) return GETM_ERR_ARG;
    const int rows = getm_tune(GETM_TUNE_COLUMN_ROWS);
    dim3 block(32, rows);
    dim3 grid(getm_div_up(a.nx_, 32), getm_div_up(a.ny_, rows));
    // the increment form's staging rings (w_substep_inc); the largest
    // carve-out of shared memory, so seven blocks of four rows fit per SM
    size_t smem = 0;
    if constexpr (getm_increment_form<V>) {
        smem = (size_t)32 * rows * w_ring_bytes_per_thread<T>();
        static bool carveout_set = false;  // a per-function attribute: once per process
        if (!carveout_set) {
            if (cudaFuncSetAttribute(wpass_kernel<T, V>, cudaFuncAttributePreferredSharedMemoryCarveout, 100) !=
                cudaSuccess)
                return GETM_ERR_CUDA;
            carveout_set = true;
        }
    }
    // Chunks: every chunk starts from h_in; the final h is the last chunk's.
    int done = 0;
    do {
        int n = ntracer - done;
        if (n > GETM_MAX_BATCH) n = GETM_MAX_BATCH;
        a.ntracer = n;
        a.h_in = h_in; a.h_out = h_out;
        for (int t = 0; t < n; t++) { a.wvar[t] = wvar[done + t]; a.f[t] = f[done + t]; }
        wpass_kernel<T, V><<<grid, block, smem, stream>>>(a);
        GETM_CHECK_LAUNCH();
        done += n;
    } while (done < ntracer);
    return GETM_OK;
}

// Fused Strang split for any form (see getm_advection_apply_3d_batch): T
// the fields, V the velocities.
template <typename T, typename V = T>
static int apply_3d_batch_impl(getm_advection* adv, getm_grid* tgrid, getm_grid* ugrid, getm_grid* vgrid,
                               int ufirst, const V* u, const V* v, const V* w, const V* const* w_var,
                               const double* Ah_u, const double* Ah_v, double timestep, double* h,
                               const double* hu, const double* hv, int ntracer, T* const* vars,
                               cudaStream_t stream)
{
    if (!adv) return GETM_OK;
    if (!tgrid || !w || !h || ntracer < 1 || !vars) return GETM_ERR_ARG;
    const int nz = tgrid->kmax - tgrid->kmin + 1;
    HPassArgs<T, V> ax, ay;
    int rc = hpass_setup<T, V>(ax, 1, adv, tgrid, ugrid, nz, u, Ah_u, 0.5 * timestep, hu);
    if (rc) return rc;
    if ((rc = hpass_setup<T, V>(ay, 2, adv, tgrid, vgrid, nz, v, Ah_v, 0.5 * timestep, hv))) return rc;
    const size_t n3 = (size_t)ax.plane * nz;
    if ((rc = adv_reserve(adv, n3, ntracer))) return rc;

    const V* wv[GETM_MAX_BATCH * 8];
    const T* fin[GETM_MAX_BATCH * 8];
    T* fout[GETM_MAX_BATCH * 8];
    T* tmp[GETM_MAX_BATCH * 8];
    for (int t = 0; t < ntracer; t++) {
        wv[t] = (w_var && w_var[t]) ? w_var[t] : w;
        tmp[t] = (T*)adv->tmp[t];
    }

    HPassArgs<T, V>* first = ufirst ? &ax : &ay;
    const int dfirst = ufirst ? 1 : 2;
    HPassArgs<T, V>* second = ufirst ? &ay : &ax;
    const int dsecond = ufirst ? 2 : 1;
    double* A = adv->hbuf[0];
    double* B = adv->hbuf[1];

    // adv1(dt/2): vars -> tmp, h -> A   (operators.py:165-170)
    for (int t = 0; t < ntracer; t++) { fin[t] = vars[t]; fout[t] = tmp[t]; }
    if ((rc = run_hstage<T, V>(*first, dfirst, h, A, ntracer, fin, fout, stream))) return rc;
    // adv2(dt/2): tmp -> vars, A -> B   (:171-175)
    for (int t = 0; t < ntracer; t++) { fin[t] = tmp[t]; fout[t] = vars[t]; }
    if ((rc = run_hstage<T, V>(*second, dsecond, A, B, ntracer, fin, fout, stream))) return rc;
    // w(dt): vars in place, B -> A      (:176-182)
    if ((rc = run_wstage<T, V>(adv, tgrid, w, wv, timestep, B, A, ntracer, vars, stream))) return rc;
    // adv2(dt/2): vars -> tmp, A -> B   (:183-188)
    for (int t = 0; t < ntracer; t++) { fin[t] = vars[t]; fout[t] = tmp[t]; }
    if ((rc = run_hstage<T, V>(*second, dsecond, A, B, ntracer, fin, fout, stream))) return rc;
    // adv1(dt/2): tmp -> vars, B -> h   (:189-193)
    for (int t = 0; t < ntracer; t++) { fin[t] = tmp[t]; fout[t] = vars[t]; }
    if ((rc = run_hstage<T, V>(*first, dfirst, B, h, ntracer, fin, fout, stream))) return rc;
    return GETM_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" int getm_advection_uv_calculate(int direction, int nk, getm_advection* adv,
                                           getm_grid* tgrid, getm_grid* ugrid, const double* u,
                                           const double* Ah, double timestep, double* h,
                                           const double* hu, double* var, cudaStream_t stream)
{
    if (!adv) return GETM_OK;  // wrapper.F90:227 returns silently without a scheme
    if ((direction != 1 && direction != 2) || nk < 1 || !h || !var) return GETM_ERR_ARG;
    HPassArgs<double> a;
    int rc = hpass_setup(a, direction, adv, tgrid, ugrid, nk, u, Ah, timestep, hu);
    if (rc) return rc;
    const size_t n3 = (size_t)a.plane * nk;
    if ((rc = adv_reserve(adv, n3, 1))) return rc;
    const double* fin[1] = {var};
    double* fout[1] = {adv->tmp[0]};
    if ((rc = run_hstage(a, direction, h, adv->hbuf[0], 1, fin, fout, stream))) return rc;
    // in-place semantics of the reference: copy the results back
    if (cudaMemcpyAsync(var, adv->tmp[0], n3 * sizeof(double), cudaMemcpyDeviceToDevice, stream) != cudaSuccess) return GETM_ERR_CUDA;
    if (cudaMemcpyAsync(h, adv->hbuf[0], n3 * sizeof(double), cudaMemcpyDeviceToDevice, stream) != cudaSuccess) return GETM_ERR_CUDA;
    return GETM_OK;
}

extern "C" int getm_advection_w_calculate(getm_advection* adv, getm_grid* tgrid, const double* w,
                                          const double* w_var, double timestep, double* h,
                                          double* var, cudaStream_t stream)
{
    if (!adv) return GETM_OK;  // wrapper.F90:265
    if (!tgrid || !w || !w_var || !h || !var || !tgrid->mask) return GETM_ERR_ARG;
    const int nz = tgrid->kmax - tgrid->kmin + 1;
    const size_t n3 = (size_t)tgrid->nx_ * tgrid->ny_ * nz;
    int rc = adv_reserve(adv, n3, 0);
    if (rc) return rc;
    const double* wv[1] = {w_var};
    double* f[1] = {var};
    if ((rc = run_wstage<double>(adv, tgrid, w, wv, timestep, h, adv->hbuf[0], 1, f, stream))) return rc;
    if (cudaMemcpyAsync(h, adv->hbuf[0], n3 * sizeof(double), cudaMemcpyDeviceToDevice, stream) != cudaSuccess) return GETM_ERR_CUDA;
    return GETM_OK;
}

extern "C" int getm_advection_apply_3d_batch(getm_advection* adv, getm_grid* tgrid,
                                             getm_grid* ugrid, getm_grid* vgrid, int ufirst,
                                             const double* u, const double* v, const double* w,
                                             const double* const* w_var, const double* Ah_u,
                                             const double* Ah_v, double timestep, double* h,
                                             const double* hu, const double* hv, int ntracer,
                                             double* const* vars, cudaStream_t stream)
{
    return apply_3d_batch_impl<double>(adv, tgrid, ugrid, vgrid, ufirst, u, v, w, w_var, Ah_u, Ah_v, timestep, h,
                                       hu, hv, ntracer, vars, stream);
}

extern "C" int getm_advection_apply_3d_batch_f32(getm_advection* adv, getm_grid* tgrid,
                                                 getm_grid* ugrid, getm_grid* vgrid, int ufirst,
                                                 const float* u, const float* v, const float* w,
                                                 const float* const* w_var, const double* Ah_u,
                                                 const double* Ah_v, double timestep, double* h,
                                                 const double* hu, const double* hv, int ntracer,
                                                 float* const* vars, cudaStream_t stream)
{
    return apply_3d_batch_impl<float>(adv, tgrid, ugrid, vgrid, ufirst, u, v, w, w_var, Ah_u, Ah_v, timestep, h,
                                      hu, hv, ntracer, vars, stream);
}

extern "C" int getm_advection_apply_3d_batch_f64s(getm_advection* adv, getm_grid* tgrid,
                                                  getm_grid* ugrid, getm_grid* vgrid, int ufirst,
                                                  const float* u, const float* v, const float* w,
                                                  const float* const* w_var, const double* Ah_u,
                                                  const double* Ah_v, double timestep, double* h,
                                                  const double* hu, const double* hv, int ntracer,
                                                  double* const* vars, cudaStream_t stream)
{
    return apply_3d_batch_impl<double, float>(adv, tgrid, ugrid, vgrid, ufirst, u, v, w, w_var, Ah_u, Ah_v,
                                              timestep, h, hu, hv, ntracer, vars, stream);
}

template <typename T, typename V = T>
static int uv_pass_impl(int direction, int nk, getm_advection* adv, getm_grid* tgrid, getm_grid* ugrid,
                        const V* u, const double* Ah, double timestep, const double* h_in, double* h_out,
                        const double* hu, int ntracer, const T* const* fin, T* const* fout, cudaStream_t stream)
{
    if (!adv || (direction != 1 && direction != 2) || nk < 1 || !h_in || !h_out || ntracer < 0) return GETM_ERR_ARG;
    if (ntracer > 0 && (!fin || !fout)) return GETM_ERR_ARG;
    if (h_in == h_out) return GETM_ERR_ARG;
    for (int t = 0; t < ntracer; t++)
        if (!fin[t] || !fout[t] || (const void*)fin[t] == (const void*)fout[t]) return GETM_ERR_ARG;
    HPassArgs<T, V> a;
    int rc = hpass_setup<T, V>(a, direction, adv, tgrid, ugrid, nk, u, Ah, timestep, hu);
    if (rc) return rc;
    return run_hstage<T, V>(a, direction, h_in, h_out, ntracer, fin, fout, stream);
}

extern "C" int getm_advection_uv_pass(int direction, int nk, getm_advection* adv, getm_grid* tgrid,
                                      getm_grid* ugrid, const double* u, const double* Ah, double timestep,
                                      const double* h_in, double* h_out, const double* hu, int ntracer,
                                      const double* const* var_in, double* const* var_out, cudaStream_t stream)
{
    return uv_pass_impl<double>(direction, nk, adv, tgrid, ugrid, u, Ah, timestep, h_in, h_out, hu, ntracer, var_in,
                                var_out, stream);
}

extern "C" int getm_advection_uv_pass_f32(int direction, int nk, getm_advection* adv, getm_grid* tgrid,
                                          getm_grid* ugrid, const float* u, const double* Ah, double timestep,
                                          const double* h_in, double* h_out, const double* hu, int ntracer,
                                          const float* const* var_in, float* const* var_out, cudaStream_t stream)
{
    return uv_pass_impl<float>(direction, nk, adv, tgrid, ugrid, u, Ah, timestep, h_in, h_out, hu, ntracer, var_in,
                               var_out, stream);
}

extern "C" int getm_advection_uv_pass_f64s(int direction, int nk, getm_advection* adv, getm_grid* tgrid,
                                           getm_grid* ugrid, const float* u, const double* Ah, double timestep,
                                           const double* h_in, double* h_out, const double* hu, int ntracer,
                                           const double* const* var_in, double* const* var_out,
                                           cudaStream_t stream)
{
    return uv_pass_impl<double, float>(direction, nk, adv, tgrid, ugrid, u, Ah, timestep, h_in, h_out, hu, ntracer,
                                       var_in, var_out, stream);
}

static int advection_2d_impl(getm_advection* adv, getm_grid* tgrid, getm_grid* ugrid, getm_grid* vgrid,
                             int ufirst, int split, const double* u, const double* v, const double* Ah_u,
                             const double* Ah_v, double timestep, double* D, const double* DU,
                             const double* DV, double* var, int increment, cudaStream_t stream)
{
    if (!adv) return GETM_OK;
    if (!D || !var || split < 1 || split > 3) return GETM_ERR_ARG;
    HPassArgs<double> ax, ay;
    int rc = hpass_setup(ax, 1, adv, tgrid, ugrid, 1, u, Ah_u, timestep, DU, increment);
    if (rc) return rc;
    if ((rc = hpass_setup(ay, 2, adv, tgrid, vgrid, 1, v, Ah_v, timestep, DV, increment))) return rc;
    const size_t n2 = (size_t)ax.plane;
    if ((rc = adv_reserve(adv, n2, 1))) return rc;
    HPassArgs<double>* p1 = ufirst ? &ax : &ay;
    HPassArgs<double>* p2 = ufirst ? &ay : &ax;
    const int d1 = ufirst ? 1 : 2, d2 = ufirst ? 2 : 1;
    double* T = adv->tmp[0];
    double* A = adv->hbuf[0];
    double* B = adv->hbuf[1];
    const double* fin[1];
    double* fout[1];
    // Sequence of (pass, dt factor); ping-pong var<->T and D->A->B->...
    int seq_n = 0;
    int seq_dir[4];
    double seq_dt[4];
    HPassArgs<double>* seq_a[4];
    if (split == 1) {          // FULL: adv1(dt), adv2(dt)
        seq_a[0] = p1; seq_dir[0] = d1; seq_dt[0] = timestep;
        seq_a[1] = p2; seq_dir[1] = d2; seq_dt[1] = timestep;
        seq_n = 2;
    } else if (split == 2) {   // HALF: adv1(dt/2), adv2(dt), adv1(dt/2)
        seq_a[0] = p1; seq_dir[0] = d1; seq_dt[0] = 0.5 * timestep;
        seq_a[1] = p2; seq_dir[1] = d2; seq_dt[1] = timestep;
        seq_a[2] = p1; seq_dir[2] = d1; seq_dt[2] = 0.5 * timestep;
        seq_n = 3;
    } else {                   // HALF_ALWAYS: adv1/2, adv2/2, adv2/2, adv1/2
        seq_a[0] = p1; seq_dir[0] = d1; seq_dt[0] = 0.5 * timestep;
        seq_a[1] = p2; seq_dir[1] = d2; seq_dt[1] = 0.5 * timestep;
        seq_a[2] = p2; seq_dir[2] = d2; seq_dt[2] = 0.5 * timestep;
        seq_a[3] = p1; seq_dir[3] = d1; seq_dt[3] = 0.5 * timestep;
        seq_n = 4;
    }
    const double* hsrc = D;
    double* fsrc = var;
    for (int s = 0; s < seq_n; s++) {
        double* hdst = (s == seq_n - 1) ? D : ((s % 2 == 0) ? A : B);
        double* fdst = (fsrc == var) ? T : var;
        seq_a[s]->dt = seq_dt[s];
        seq_a[s]->dtf = (float)seq_dt[s];
        fin[0] = fsrc; fout[0] = fdst;
        if ((rc = run_hstage(*seq_a[s], seq_dir[s], hsrc, hdst, 1, fin, fout, stream))) return rc;
        hsrc = hdst;
        fsrc = fdst;
    }
    if (fsrc != var) {
        if (cudaMemcpyAsync(var, fsrc, n2 * sizeof(double), cudaMemcpyDeviceToDevice, stream) != cudaSuccess) return GETM_ERR_CUDA;
    }
    return GETM_OK;
}

int getm_advection_2d_passes(getm_advection* adv, getm_grid* tgrid, getm_grid* ugrid, getm_grid* vgrid,
                             int ufirst, const double* u, const double* v, double timestep, double* D,
                             const double* DU, const double* DV, double* var, int increment,
                             Advection2DPasses* out)
{
    if (!adv || !D || !var || !out) return GETM_ERR_ARG;
    HPassArgs<double> ax, ay;
    int rc = hpass_setup(ax, 1, adv, tgrid, ugrid, 1, u, nullptr, timestep, DU, increment);
    if (rc) return rc;
    if ((rc = hpass_setup(ay, 2, adv, tgrid, vgrid, 1, v, nullptr, timestep, DV, increment))) return rc;
    if ((rc = adv_reserve(adv, (size_t)ax.plane, 1))) return rc;
    out->pass[0] = ufirst ? ax : ay;
    out->pass[1] = ufirst ? ay : ax;
    out->dir[0] = ufirst ? 1 : 2;
    out->dir[1] = ufirst ? 2 : 1;
    HPassArgs<double>& p1 = out->pass[0];
    HPassArgs<double>& p2 = out->pass[1];
    p1.ntracer = p2.ntracer = 1;
    p1.h_in = D; p1.h_out = adv->hbuf[0]; p1.fin[0] = var; p1.fout[0] = adv->tmp[0];
    p2.h_in = adv->hbuf[0]; p2.h_out = D; p2.fin[0] = adv->tmp[0]; p2.fout[0] = var;
    return GETM_OK;
}

extern "C" int getm_advection_2d(getm_advection* adv, getm_grid* tgrid, getm_grid* ugrid,
                                 getm_grid* vgrid, int ufirst, int split, const double* u,
                                 const double* v, const double* Ah_u, const double* Ah_v,
                                 double timestep, double* D, const double* DU, const double* DV,
                                 double* var, cudaStream_t stream)
{
    return advection_2d_impl(adv, tgrid, ugrid, vgrid, ufirst, split, u, v, Ah_u, Ah_v, timestep, D, DU, DV, var,
                             0, stream);
}

extern "C" int getm_advection_2d_mixed(getm_advection* adv, getm_grid* tgrid, getm_grid* ugrid,
                                       getm_grid* vgrid, int ufirst, int split, const double* u,
                                       const double* v, const double* Ah_u, const double* Ah_v,
                                       double timestep, double* D, const double* DU, const double* DV,
                                       double* var, cudaStream_t stream)
{
    return advection_2d_impl(adv, tgrid, ugrid, vgrid, ufirst, split, u, v, Ah_u, Ah_v, timestep, D, DU, DV, var,
                             1, stream);
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the 2D advection split
// ---------------------------------------------------------------------------
// getm_advection_2d keeps its ping-pong buffers in a handle that allocates
// them with cudaMalloc on first use.  Some callers cannot allow that: a host
// model that hands all device memory to its own pool allocator at start-up
// (a library cudaMalloc then fails or breaks the pool's accounting), and
// drivers that must not let a library call synchronize the device (cudaMalloc
// and cudaFree may do so implicitly).  getm_advection_2d_noalloc takes the
// scheme instead of a handle and keeps its three work buffers (tracer
// ping-pong copy and two column-height buffers) in one file-scope device
// array of fixed size, so it allocates nothing.
//
// Limits and sharing rules:
// * the domain may have at most GETM_NOALLOC_MAX_POINTS points including
//   halos (nx_ * ny_); larger domains get GETM_ERR_TOO_LARGE and nothing runs;
// * every GPU that loads the library holds the 3 * 2^20 doubles (24 MiB)
//   until the process exits;
// * all calls share the one array, which keeps the previous call's contents.
//   Nothing in it has to start at zero: every pass writes all points of the
//   buffer it produces before the next pass reads them.  Calls that overlap on
//   the GPU (different streams, or different host threads without ordering)
//   race on the array and corrupt each other's results;
// * the first call on a device looks up the array's device address with
//   cudaGetSymbolAddress (once per device, with that device current).  Make
//   that first call before any stream capture.
#include <mutex>

#define GETM_NOALLOC_MAX_POINTS (1 << 20)
#define GETM_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_noalloc_scratch[3 * GETM_NOALLOC_MAX_POINTS];
static double* g_noalloc_ptr[GETM_NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mutex;

// Device address of the scratch array for the current device.
static int noalloc_scratch(double** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GETM_ERR_CUDA;
    if (dev < 0 || dev >= GETM_NOALLOC_MAX_DEVICES) return GETM_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = NULL;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == NULL) return GETM_ERR_CUDA;
        g_noalloc_ptr[dev] = (double*)p;
    }
    *out = g_noalloc_ptr[dev];
    return GETM_OK;
}

extern "C" int getm_advection_2d_noalloc(int scheme, getm_grid* tgrid, getm_grid* ugrid, getm_grid* vgrid,
                                         int ufirst, int split, const double* u, const double* v,
                                         const double* Ah_u, const double* Ah_v, double timestep, double* D,
                                         const double* DU, const double* DV, double* var, cudaStream_t stream)
{
    if (scheme < GETM_SCHEME_HSIMT || scheme > GETM_SCHEME_UPSTREAM) return GETM_ERR_ARG;
    if (!tgrid || !D || !var || split < 1 || split > 3) return GETM_ERR_ARG;
    const long long npoints = (long long)tgrid->nx_ * tgrid->ny_;
    if (npoints > GETM_NOALLOC_MAX_POINTS) return GETM_ERR_TOO_LARGE;
    getm_advection adv;  // scheme only: lives on the host stack, owns nothing
    memset(&adv, 0, sizeof(adv));
    adv.scheme = scheme;
    HPassArgs<double> ax, ay;
    int rc = hpass_setup(ax, 1, &adv, tgrid, ugrid, 1, u, Ah_u, timestep, DU);
    if (rc) return rc;
    if ((rc = hpass_setup(ay, 2, &adv, tgrid, vgrid, 1, v, Ah_v, timestep, DV))) return rc;
    double* scratch = NULL;
    if ((rc = noalloc_scratch(&scratch))) return rc;
    double* T = scratch;
    double* A = scratch + GETM_NOALLOC_MAX_POINTS;
    double* B = scratch + 2 * GETM_NOALLOC_MAX_POINTS;
    HPassArgs<double>* p1 = ufirst ? &ax : &ay;
    HPassArgs<double>* p2 = ufirst ? &ay : &ax;
    const int d1 = ufirst ? 1 : 2, d2 = ufirst ? 2 : 1;
    int seq_n = 0;
    int seq_dir[4];
    double seq_dt[4];
    HPassArgs<double>* seq_a[4];
    if (split == 1) {  // FULL (operators.py:76-79)
        seq_a[0] = p1; seq_dir[0] = d1; seq_dt[0] = timestep;
        seq_a[1] = p2; seq_dir[1] = d2; seq_dt[1] = timestep;
        seq_n = 2;
    } else if (split == 2) {  // HALF (operators.py:80-85)
        seq_a[0] = p1; seq_dir[0] = d1; seq_dt[0] = 0.5 * timestep;
        seq_a[1] = p2; seq_dir[1] = d2; seq_dt[1] = timestep;
        seq_a[2] = p1; seq_dir[2] = d1; seq_dt[2] = 0.5 * timestep;
        seq_n = 3;
    } else {  // HALF_ALWAYS (operators.py:86-93)
        seq_a[0] = p1; seq_dir[0] = d1; seq_dt[0] = 0.5 * timestep;
        seq_a[1] = p2; seq_dir[1] = d2; seq_dt[1] = 0.5 * timestep;
        seq_a[2] = p2; seq_dir[2] = d2; seq_dt[2] = 0.5 * timestep;
        seq_a[3] = p1; seq_dir[3] = d1; seq_dt[3] = 0.5 * timestep;
        seq_n = 4;
    }
    const double* fin[1];
    double* fout[1];
    const double* hsrc = D;
    double* fsrc = var;
    for (int s = 0; s < seq_n; s++) {
        double* hdst = (s == seq_n - 1) ? D : ((s % 2 == 0) ? A : B);
        double* fdst = (fsrc == var) ? T : var;
        seq_a[s]->dt = seq_dt[s];
        seq_a[s]->dtf = (float)seq_dt[s];
        fin[0] = fsrc;
        fout[0] = fdst;
        if ((rc = run_hstage(*seq_a[s], seq_dir[s], hsrc, hdst, 1, fin, fout, stream))) return rc;
        hsrc = hdst;
        fsrc = fdst;
    }
    if (fsrc != var) {
        if (cudaMemcpyAsync(var, fsrc, (size_t)npoints * sizeof(double), cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
            return GETM_ERR_CUDA;
    }
    return GETM_OK;
}
