/*
 * getm_gb300: C ABI of the GB300 (sm_103a) implementation of pygetm's
 * split-explicit time-step operators.
 *
 * Every entry point mirrors one bind(c) routine of the reference Fortran
 * library (declared to Cython at python/_pygetm.pyx:24-66) with the same
 * argument list and meaning, and adds:
 *   - all array arguments are DEVICE pointers (C layout [k][j][i], i fastest,
 *     halos included, exactly as pygetm passes them);
 *   - a trailing cudaStream_t on which the work is enqueued (stream-ordered,
 *     no host synchronisation);
 *   - an int status return (GETM_OK = 0) instead of a void return; the
 *     reference aborts or silently returns where these return an error code.
 * Functions named *_f32 are the mixed-precision form: bulk fields in float,
 * layer thicknesses and elevations in double.
 * Index bounds (imin..jmax) are the reference's Fortran 1-based ones.
 */
#ifndef GETM_GB300_H
#define GETM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#ifndef __CUDA_RUNTIME_H__
typedef struct CUstream_st* cudaStream_t;
#endif

/* status codes */
#define GETM_OK 0
#define GETM_ERR_ARG 1          /* null pointer, bad extent or unknown name */
#define GETM_ERR_CUDA 2         /* a CUDA launch/runtime call failed */
#define GETM_ERR_ITERS 3        /* vertical advection hit itersmax (200) sub-steps */
#define GETM_ERR_NZ 4           /* more layers than a column kernel supports */
#define GETM_ERR_ALLOC 5        /* device work-buffer allocation failed */
#define GETM_ERR_TOO_LARGE 6    /* domain exceeds the fixed scratch of an allocation-free call */

/* advection schemes: src/operators/advection.F90:22-30 */
#define GETM_SCHEME_HSIMT 1
#define GETM_SCHEME_MUSCL 2
#define GETM_SCHEME_P2_PDM 3
#define GETM_SCHEME_SPLMAX13 4
#define GETM_SCHEME_SUPERBEE 5
#define GETM_SCHEME_UPSTREAM 6

/* largest number of layers the column kernels (vertical advection and
 * diffusion) accept */
#define GETM_MAX_NZ 256
/* tracers per getm_domain_totals call, and blocks of its first stage (the
 * work buffer holds 2 * GETM_TOTALS_BLOCKS * (1 + ntracer) doubles) */
#define GETM_MAX_TOTALS 16
#define GETM_TOTALS_BLOCKS 608

typedef struct getm_grid getm_grid;
typedef struct getm_advection getm_advection;
typedef struct getm_vertical_diffusion getm_vertical_diffusion;

/* ---- grids --------------------------------------------------------------
 * create_grid: python/src/wrapper.F90:48-59 (pyx:26)
 * grid_finalize: wrapper.F90:61-68 (pyx:27)
 * getm_grid_set_array replaces get_array (wrapper.F90:70-125, pyx:34): the
 * reference grid owns its metric arrays and hands out pointers to them; here
 * the caller owns the device storage and registers it by the same names
 * ("mask", "dx", "dy", "idx", "idy", "iarea", "area").                        */
int getm_create_grid(int imin, int imax, int jmin, int jmax, int kmin, int kmax, int halox,
                     int haloy, getm_grid** grid);
int getm_grid_finalize(getm_grid* grid);
int getm_grid_set_array(getm_grid* grid, const char* name, void* device_ptr);
/* No counterpart in the reference (it has no float arithmetic).  The float
 * copies of a grid's registered metrics, which the mixed form's kernels read,
 * converted on `stream` after the metrics' earlier writes on that stream;
 * returns when `stream` has finished them and waits for no other stream.
 * Without this call the first float kernel on the grid makes them, and that
 * first use waits for the whole device.                                       */
int getm_grid_float_metrics(getm_grid* grid, cudaStream_t stream);

/* ---- advection ----------------------------------------------------------
 * advection_create/finalize: wrapper.F90:188-211 (pyx:35-36)
 * advection_uv_calculate: wrapper.F90:213-254 (pyx:37); direction 1 = x
 *   (ugrid mask/idx/dy), 2 = y (vgrid mask/dx/idy); Ah == NULL: no diffusion.
 * advection_w_calculate: wrapper.F90:256-273 (pyx:38).                      */
int getm_advection_create(int scheme, getm_grid* tgrid, getm_advection** adv);
int getm_advection_finalize(getm_advection* adv);
int getm_advection_uv_calculate(int direction, int nk, getm_advection* adv, getm_grid* tgrid,
                                getm_grid* ugrid, const double* u, const double* Ah,
                                double timestep, double* h, const double* hu, double* var,
                                cudaStream_t stream);
int getm_advection_w_calculate(getm_advection* adv, getm_grid* tgrid, const double* w,
                               const double* w_var, double timestep, double* h, double* var,
                               cudaStream_t stream);
/* Fused 3D Strang split of python/pygetm/operators.py:135-193
 * (Advection.apply_3d_batch; apply_3d is ntracer == 1): adv1(dt/2),
 * adv2(dt/2), w(dt), adv2(dt/2), adv1(dt/2) with adv1 = v unless ufirst, for
 * ntracer tracers sharing one evolving layer thickness h (in/out).  w_var[t]
 * may equal w.  ugrid/vgrid metrics come from the grid handles.              */
int getm_advection_apply_3d_batch(getm_advection* adv, getm_grid* tgrid, getm_grid* ugrid,
                                  getm_grid* vgrid, int ufirst, const double* u,
                                  const double* v, const double* w, const double* const* w_var,
                                  const double* Ah_u, const double* Ah_v, double timestep,
                                  double* h, const double* hu, const double* hv, int ntracer,
                                  double* const* vars, cudaStream_t stream);
/* One directional pass of advection_uv_calculate (wrapper.F90:213-254),
 * out of place and batched: reads h_in and var_in[t], writes the complete
 * fields h_out and var_out[t] (every point; untouched points are copied).
 * One kernel launch for up to 32 tracers.  Buffers must not alias.          */
int getm_advection_uv_pass(int direction, int nk, getm_advection* adv, getm_grid* tgrid,
                           getm_grid* ugrid, const double* u, const double* Ah, double timestep,
                           const double* h_in, double* h_out, const double* hu, int ntracer,
                           const double* const* var_in, double* const* var_out, cudaStream_t stream);
/* Fused 2D split of Advection.__call__ (operators.py:52-93): split 1 = FULL,
 * 2 = HALF, 3 = HALF_ALWAYS; D (in/out) is the column-height work array.    */
int getm_advection_2d(getm_advection* adv, getm_grid* tgrid, getm_grid* ugrid, getm_grid* vgrid,
                      int ufirst, int split, const double* u, const double* v,
                      const double* Ah_u, const double* Ah_v, double timestep, double* D,
                      const double* DU, const double* DV, double* var, cudaStream_t stream);
/* Allocation-free 2D split.  No counterpart in the reference: it is
 * getm_advection_2d for callers that cannot let the library call cudaMalloc
 * (a host model whose pool allocator owns all device memory, or a driver that
 * must not let a library call synchronize the device).  Takes the scheme
 * instead of an advection handle and keeps its work buffers in a fixed
 * file-scope device array: at most 1048576 points (nx_*ny_, halos included),
 * else GETM_ERR_TOO_LARGE; 24 MiB held per GPU until exit.  All calls share
 * that array: calls that overlap on the GPU race.  The first call on a device
 * looks up the array's address (cudaGetSymbolAddress) and should come before
 * any stream capture.                                                        */
int getm_advection_2d_noalloc(int scheme, getm_grid* tgrid, getm_grid* ugrid, getm_grid* vgrid,
                              int ufirst, int split, const double* u, const double* v,
                              const double* Ah_u, const double* Ah_v, double timestep, double* D,
                              const double* DU, const double* DV, double* var, cudaStream_t stream);
/* Status word of the last vertical advection on this handle's stream:
 * GETM_ERR_ITERS if a column needed more than itersmax sub-steps.  Blocks
 * until the handle's pending work on `stream` is done.                      */
int getm_advection_get_status(getm_advection* adv, cudaStream_t stream);

/* ---- vertical diffusion -------------------------------------------------
 * vertical_diffusion_create/finalize: wrapper.F90:127-147 (pyx:39-40)
 * c_vertical_diffusion_prepare: wrapper.F90:149-161 -> diffusion.F90:135-204
 * c_vertical_diffusion_apply: wrapper.F90:163-186 -> diffusion.F90:206-314
 * nuh has nz+1 interface levels; ea2/ea4 may be NULL.                       */
int getm_vertical_diffusion_create(getm_grid* tgrid, getm_vertical_diffusion** diff);
int getm_vertical_diffusion_finalize(getm_vertical_diffusion* diff);
int getm_vertical_diffusion_prepare(getm_vertical_diffusion* diff, int nx, int ny, int nz,
                                    double molecular, const double* nuh, double timestep,
                                    double cnpar, const int* mask, const double* ho,
                                    const double* hn, cudaStream_t stream);
int getm_vertical_diffusion_apply(getm_vertical_diffusion* diff, int nx, int ny, int nz,
                                  const int* mask, const double* ho, const double* hn,
                                  double* var, const double* ea2, const double* ea4,
                                  cudaStream_t stream);
/* prepare + apply fused per column (VerticalDiffusion.__call__,
 * operators.py:218-230) for ntracer fields, each with its own molecular
 * diffusivity and optional ea2/ea4 (arrays of device pointers, entries may be
 * NULL; the arrays themselves may be NULL).  work: NULL (elimination
 * coefficients in shared memory) or a device buffer of 2*nx*ny*nz elements
 * of the field type (more columns resident per SM); the _f32 form solves
 * its fields in pairs and needs 4*nx*ny*nz elements when ntracer > 1.       */
int getm_vertical_diffusion_batch(int nx, int ny, int nz, const int* mask, const double* nuh,
                                  double timestep, double cnpar, const double* ho,
                                  const double* hn, int ntracer, const double* molecular,
                                  double* const* vars, const double* const* ea2,
                                  const double* const* ea4, double* work, cudaStream_t stream);

/* ---- python/src/interpolation.F90:9-72 (pyx:28-31) ---------------------- */
int getm_grid_interp_x(int nx, int ny, int nz, const double* source, double* target, int ioffset,
                       cudaStream_t stream);
int getm_grid_interp_y(int nx, int ny, int nz, const double* source, double* target, int joffset,
                       cudaStream_t stream);
int getm_grid_interp_z(int nx, int ny, int nz1, int nz2, const double* source, double* target,
                       int koffset, cudaStream_t stream);
int getm_grid_interp_xy(int nx1, int ny1, int nx2, int ny2, int nz, const double* source,
                        double* target, int ioffset, int joffset, cudaStream_t stream);

/* ---- python/src/wrapper.F90 --------------------------------------------- */
/* c_momentum_diffusion: wrapper.F90:275-393 (pyx:43) */
int getm_momentum_diffusion(getm_grid* ugrid, getm_grid* vgrid, getm_grid* uugrid,
                            getm_grid* uvgrid, getm_grid* vugrid, getm_grid* vvgrid, int nk,
                            const double* huu, const double* huv, const double* hvu,
                            const double* hvv, const double* u, const double* v, double Am0,
                            double* diffu, double* diffv, cudaStream_t stream);
/* c_thickness2center_depth: wrapper.F90:395-407 (pyx:46) */
int getm_thickness2center_depth(int nx, int ny, int nz, int istart, int istop, int jstart,
                                int jstop, const int* mask, const double* h, double* out,
                                cudaStream_t stream);
/* c_thickness2vertical_coordinates: wrapper.F90:409-426 (pyx:47) */
int getm_thickness2vertical_coordinates(int nx, int ny, int nz, const int* mask,
                                        const double* bottom_depth, const double* h, double* zc,
                                        double* zf, cudaStream_t stream);
/* c_alpha: wrapper.F90:428-435 (pyx:48) */
int getm_alpha(int n, const double* D, double Dmin, double Dcrit, const int* mask, double* alpha,
               cudaStream_t stream);
/* c_elevation2depth: wrapper.F90:437-445 (pyx:49) */
int getm_elevation2depth(int n, const double* z, const double* H, double Dmin, const int* mask,
                         double* D, cudaStream_t stream);
/* c_vertical_advection_to_sources: wrapper.F90:447-485 (pyx:65, 574-575):
 * first-order upstream vertical fluxes of c (w at the layer centres, levels
 * surface to bottom, mask 3D) added to the source term s; nothing changes
 * when w is zero at every interior point.  work: one int of device memory
 * (the test's flag).                                                      */
int getm_vertical_advection_to_sources(int nx, int ny, int nz, int halox, int haloy, const int* mask,
                                       const double* c, const double* w, const double* h, double* s,
                                       int* work, cudaStream_t stream);
/* c_update_gvc: wrapper.F90:567-600 (pyx:66, 577-585): general vertical
 * coordinates; layer thicknesses h (nz x ny x nx) where mask != 0 from the
 * water depth D, the equidistant fraction dsigma, the zoomed fractions
 * dbeta (nz values, device memory), Dgamma and the 1-based reference
 * layer kk.                                                               */
int getm_update_gvc(int nx, int ny, int nz, double dsigma, const double* dbeta, double Dgamma, int kk,
                    const double* D, const int* mask, double* h, cudaStream_t stream);
/* c_multiply_add: wrapper.F90:488-494 (pyx:60) */
int getm_multiply_add(int n, double* tgt, const double* add, double scale_factor,
                      cudaStream_t stream);
/* c_advance_surface_elevation: wrapper.F90:496-523 (pyx:61) */
int getm_advance_surface_elevation(int nx, int ny, int halox, int haloy, const int* mask,
                                   const double* dyu, const double* dxv, const double* iarea,
                                   double* z, const double* U, const double* V,
                                   const double* fwf, double dt, cudaStream_t stream);
/* c_surface_pressure_gradient: wrapper.F90:525-565 (pyx:62) */
int getm_surface_pressure_gradient(int nx, int ny, int imin, int imax, int jmin, int jmax,
                                   const int* umask, const int* vmask, const double* idxu,
                                   const double* idyv, const double* z, const double* sp,
                                   const double* H, const double* D, double Dmin, double* dpdx,
                                   double* dpdy, cudaStream_t stream);
/* The same, mixed form: elevation bounds compared on the integer pipe, the
 * elevation and air-pressure differences in FP64, the rest in float (the
 * mixed transport update reads the gradient as a float).                   */
int getm_surface_pressure_gradient_mixed(int nx, int ny, int imin, int imax, int jmin, int jmax,
                                         const int* umask, const int* vmask, const double* idxu,
                                         const double* idyv, const double* z, const double* sp,
                                         const double* H, const double* D, double Dmin, double* dpdx,
                                         double* dpdy, cudaStream_t stream);

/* ---- python/src/momentum.F90 --------------------------------------------- */
/* c_horizontal_diffusion: momentum.F90:12-77 (pyx:50) */
int getm_horizontal_diffusion(int imin, int imax, int jmin, int jmax, int halox, int haloy,
                              const int* umask, const int* vmask, const double* idxu,
                              const double* dyu, const double* idyv, const double* dxv,
                              const double* Ah_u, const double* Ah_v, const int* tmask,
                              const double* iA, double dt, const double* f, double* out,
                              cudaStream_t stream);
/* c_bottom_friction: momentum.F90:79-101 (pyx:51) */
int getm_bottom_friction(int nx, int ny, const int* mask, const double* u, const double* v,
                         const double* D, double* z0b, const double* z0b_in, double avmmol,
                         double* ru, int iterate, cudaStream_t stream);
/* c_collect_3d_momentum_sources: momentum.F90:103-145 (pyx:52) */
int getm_collect_3d_momentum_sources(int nx, int ny, int nz, int halox, int haloy,
                                     const int* mask, const double* alpha, const double* ho,
                                     const double* hn, const double* dp, const double* cor,
                                     const double* adv, const double* diff, const double* idp,
                                     const double* taus, const double* rr, double dt,
                                     double* ea2, double* ea4, cudaStream_t stream);
/* c_advance_2d_transport: momentum.F90:147-189 (pyx:53) */
int getm_advance_2d_transport(int nx, int ny, int halox, int haloy, const int* mask,
                              const double* alpha, const double* D, const double* dp,
                              const double* taus, const double* cor, const double* adv,
                              const double* diff, const double* damp, const double* SA,
                              const double* SB, const double* SD, const double* SF,
                              const double* r, double dt, double* U, cudaStream_t stream);
/* c_w_momentum_3d: momentum.F90:191-216 (pyx:54) */
int getm_w_momentum_3d(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                       const int* mask, const double* dyu, const double* dxv,
                       const double* iarea, const double* ho, const double* hn,
                       const double* pk, const double* qk, double dt, double* w,
                       cudaStream_t stream);
/* c_shear_frequency: momentum.F90:218-241 (pyx:55) */
int getm_shear_frequency(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                         const int* mask, const double* hu, const double* hv, const double* uk,
                         const double* vk, double* SS, cudaStream_t stream);
/* c_shear_frequency2: momentum.F90:244-268 (pyx:56, 468-479): the squared
 * shear frequency weighted by the viscosity num at the four neighbouring
 * velocity points, over num at the T point; h, hu, hv layer thicknesses of
 * the T, U, V grids.  _f32: float uk, vk, num, SS.                          */
int getm_shear_frequency2(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax, const int* mask,
                          const double* h, const double* hu, const double* hv, const double* uk,
                          const double* vk, const double* num, double* SS, cudaStream_t stream);
int getm_shear_frequency2_f32(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax, const int* mask,
                              const double* h, const double* hu, const double* hv, const float* uk,
                              const float* vk, const float* num, float* SS, cudaStream_t stream);
/* c_surface_shear_velocity: momentum.F90:270-284 (pyx:57) */
int getm_surface_shear_velocity(int nx, int ny, int imin, int imax, int jmin, int jmax,
                                const int* mask, const double* tausx, const double* tausy,
                                double* ustar2_s, cudaStream_t stream);
/* c_bottom_shear_velocity: momentum.F90:286-321 (pyx:58) */
int getm_bottom_shear_velocity(int nx, int ny, int imin, int imax, int jmin, int jmax,
                               const int* mask, const int* umask, const int* vmask,
                               const double* uk_bot, const double* vk_bot, const double* rru,
                               const double* rrv, double* taubx, double* tauby,
                               double* ustar2_b, cudaStream_t stream);
/* c_reconstruct_transport_change: momentum.F90:323-340 (pyx:59) */
int getm_reconstruct_transport_change(int nx, int ny, int nz, int imin, int imax, int jmin,
                                      int jmax, double* un, const double* hn, const double* Uo,
                                      double timestep, cudaStream_t stream);

/* ---- python/src/internal_pressure.F90 ----------------------------------- */
/* c_blumberg_mellor: internal_pressure.F90:9-60 (pyx:63) */
int getm_blumberg_mellor(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                         const int* umask, const int* vmask, const double* idxu,
                         const double* idyv, const double* hu, const double* hv,
                         const double* zf, const double* buoy, double* idpdx, double* idpdy,
                         cudaStream_t stream);
/* c_shchepetkin_mcwilliams: internal_pressure.F90:63-217 (pyx:64).
 * P_work: caller-provided device scratch of nx*ny*nz doubles (the
 * reference allocates dR, dZ, P per call).                                  */
int getm_shchepetkin_mcwilliams(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                                const int* mask, const int* umask, const int* vmask,
                                const double* idxu, const double* idyv, const double* h,
                                const double* z, const double* zc, const double* buoy,
                                double* idpdx, double* idpdy, double* P_work,
                                cudaStream_t stream);

/* ---- instrumentation ----------------------------------------------------
 * No counterpart in the reference.  Number of kernel launches this library
 * has issued in the process so far (launches captured into a CUDA graph are
 * counted once, at capture).                                                */
int getm_launch_count(unsigned long long* count);

/* No counterpart in the reference.  Launch an instantiated CUDA graph
 * (cudaGraphExec_t, e.g. a domain's recorded 3D step) on `stream`.  Unlike
 * PyTorch's CUDAGraph.replay, this may be called by one host thread while
 * another captures a graph in thread-local mode (serving: steps of running
 * requests keep being issued while a new request is recorded).            */
int getm_graph_launch(void* graph_exec, cudaStream_t stream);

/* The model time of a substep that is not the one-launch substep (which
 * advances it itself): *time += timestep on the device, so that a captured
 * step graph advances it too.  pygetm keeps its time on the host
 * (python/pygetm/simulation.py:291-325, self.time += self.timestep).      */
int getm_advance_time(double* time, double timestep, cudaStream_t stream);

/* No counterpart in the reference.  A stream of the calling thread's current
 * device that belongs to the caller alone (non-blocking; priority as in
 * cudaStreamCreateWithPriority).  PyTorch's torch.cuda.Stream() hands out
 * streams from a small shared pool, so two of them can be the same CUDA
 * stream: a stream that one thread issues graph launches on must not be one
 * that another thread's capture has drawn in.                               */
int getm_stream_create(int priority, cudaStream_t* stream);
int getm_stream_destroy(cudaStream_t stream);

/* ---- launch-shape knobs (the autotuner's search space) -----------------
 * No counterpart in the reference.  Launch shapes of the hot kernels, read
 * on the calling host thread at every launch (a CUDA graph keeps the shapes
 * it was captured with).  The table is per host thread and starts at the
 * defaults; a value outside the knob's set returns GETM_ERR_ARG.
 *   GETM_TUNE_XPASS_ROWS      rows (warps) per block of the x pass: 2, 4, 8 (default 8)
 *   GETM_TUNE_YMARCH_CHUNK    rows a warp marches in the 3D y pass: 16, 32, 64 (default 32)
 *   GETM_TUNE_COLUMN_ROWS     rows of 32 columns per block of the w pass and
 *                             the float column solve: 1, 2, 4 (default 4)
 *   GETM_TUNE_SUBSTEP_BLOCKS  blocks per SM of the one-launch 2D substep:
 *                             0 = as many as fit (default), 1, 2 (capped at what fits)
 *   GETM_TUNE_XPASS_VEC       3D x pass in increment form: 1 = four cells per lane
 *                             where rows allow 16-byte vectors (default), 0 = one
 *                             cell per lane (both give the same bits)
 *   GETM_TUNE_COLUMN_SOLVE    float column solve (mixed form): 0 = one thread per
 *                             column (default), 1 = four warps per 32 columns, each
 *                             owning a quarter of the levels (partition method),
 *                             for 8 <= nz <= 64.  Unlike the other knobs this one
 *                             changes the rounding of the solve's increments.   */
#define GETM_TUNE_XPASS_ROWS 0
#define GETM_TUNE_YMARCH_CHUNK 1
#define GETM_TUNE_COLUMN_ROWS 2
#define GETM_TUNE_SUBSTEP_BLOCKS 3
#define GETM_TUNE_XPASS_VEC 4
#define GETM_TUNE_COLUMN_SOLVE 5
#define GETM_TUNE_NKNOBS 6
int getm_tune_set(int knob, int value);
int getm_tune_get(int knob, int* value);

/* ---- equation of state --------------------------------------------------
 * No counterpart in the reference's Fortran: pygetm takes density from the
 * external TEOS-10 package pygsw (python/pygetm/density.py:62-95).  This
 * device EOS is the simplified nonlinear equation of state of Roquet et al.
 * (2015); p is depth below the surface (m).  Writes rho and/or buoyancy
 * -g/rho0 (rho - rho0) (python/pygetm/simulation.py:1184); either may be NULL. */
int getm_density_buoyancy(int n, const double* salt, const double* temp, const double* p, double* rho,
                          double* buoy, cudaStream_t stream);

/* Momentum.advance (momentum.py:790-793): Ui = U_cum * scale, Vi = V_cum *
 * scale (scale = 1 / split_factor), then U_cum = V_cum = 0; n points.      */
int getm_mean_transports(long long n, double* Ucum, double* Vcum, double scale, double* Ui, double* Vi,
                         cudaStream_t stream);
/* Momentum.update_diagnostics (momentum.py:1003-1015): SxF = ustar2_bx +
 * ru * u1 and SyF = ustar2_by + rv * v1 (product and sum rounded
 * separately), n points.                                                   */
int getm_slow_friction(long long n, const double* ustar2x, const double* ru, const double* u1, double* SxF,
                       const double* ustar2y, const double* rv, const double* v1, double* SyF, cudaStream_t stream);

/* ---- mixed-precision form ------------------------------------------------
 * Same routines with float bulk fields (tracers, 3D velocities/transports,
 * their tendencies, nuh/num) and float arithmetic for fluxes, limiters and
 * the tridiagonal solves.  Layer thicknesses, elevations, water depths,
 * metrics, 2D transports, density, buoyancy and the internal pressure
 * gradient stay double (the gradient is a small difference of large column
 * integrals of buoyancy); the thickness updates and the w recursion are
 * evaluated in FP64, the momentum sources in float.  The *_f32 internal-pressure
 * entry points (float buoyancy and gradients) remain available.           */
int getm_advection_apply_3d_batch_f32(getm_advection* adv, getm_grid* tgrid, getm_grid* ugrid,
                                      getm_grid* vgrid, int ufirst, const float* u, const float* v,
                                      const float* w, const float* const* w_var, const double* Ah_u,
                                      const double* Ah_v, double timestep, double* h,
                                      const double* hu, const double* hv, int ntracer,
                                      float* const* vars, cudaStream_t stream);
int getm_advection_uv_pass_f32(int direction, int nk, getm_advection* adv, getm_grid* tgrid,
                               getm_grid* ugrid, const float* u, const double* Ah, double timestep,
                               const double* h_in, double* h_out, const double* hu, int ntracer,
                               const float* const* var_in, float* const* var_out, cudaStream_t stream);
int getm_vertical_diffusion_batch_f32(int nx, int ny, int nz, const int* mask, const float* nuh,
                                      double timestep, double cnpar, const double* ho,
                                      const double* hn, int ntracer, const double* molecular,
                                      float* const* vars, const float* const* ea2,
                                      const float* const* ea4, float* work, cudaStream_t stream);
/* The mixed form with FP64 tracer storage: fields (tracers) double, every
 * other operand as in the _f32 entries (float velocities, w, nuh, sources
 * and work); the increments, fluxes, limiters and the solve are float, the
 * differences of neighbouring values are formed in FP64 before they are
 * narrowed, and each field is updated in FP64 (value + float increment).
 * Same arguments as getm_advection_apply_3d_batch_f32 and
 * getm_vertical_diffusion_batch_f32 otherwise.                             */
int getm_advection_apply_3d_batch_f64s(getm_advection* adv, getm_grid* tgrid, getm_grid* ugrid,
                                       getm_grid* vgrid, int ufirst, const float* u, const float* v,
                                       const float* w, const float* const* w_var, const double* Ah_u,
                                       const double* Ah_v, double timestep, double* h,
                                       const double* hu, const double* hv, int ntracer,
                                       double* const* vars, cudaStream_t stream);
/* getm_velocities_3d_f32, also writing the bottom layer (the first `plane`
 * points) of uk and vk widened to double into ubot, vbot (the FP64 bottom
 * velocities of the mixed form's 2D friction).                             */
int getm_velocities_3d_bottom_f32(long long n, long long plane, const float* pk, const double* hnu,
                                  const float* qk, const double* hnv, float* uk, float* vk, double* ubot,
                                  double* vbot, cudaStream_t stream);
/* Density and buoyancy from FP64 S and T with the mixed form's arithmetic
 * (the double-float anomaly of getm_density_buoyancy_f32, each input split
 * into two floats); the squared buoyancy frequency from FP64 S and T in
 * float arithmetic (temperature and salinity differences formed in FP64),
 * float NN.                                                                 */
int getm_density_buoyancy_f64s(int n, const double* salt, const double* temp, const double* p, double* rho,
                               double* buoy, cudaStream_t stream);
int getm_buoyancy_frequency_f64s(int nx, int ny, int nz, const int* mask, const double* h, const double* p,
                                 const double* salt, const double* temp, float* NN, cudaStream_t stream);
int getm_advection_uv_pass_f64s(int direction, int nk, getm_advection* adv, getm_grid* tgrid,
                                getm_grid* ugrid, const float* u, const double* Ah, double timestep,
                                const double* h_in, double* h_out, const double* hu, int ntracer,
                                const double* const* var_in, double* const* var_out, cudaStream_t stream);
int getm_vertical_diffusion_batch_f64s(int nx, int ny, int nz, const int* mask, const float* nuh,
                                       double timestep, double cnpar, const double* ho,
                                       const double* hn, int ntracer, const double* molecular,
                                       double* const* vars, const float* const* ea2,
                                       const float* const* ea4, float* work, cudaStream_t stream);
int getm_grid_interp_x_f32(int nx, int ny, int nz, const float* source, float* target, int ioffset,
                           cudaStream_t stream);
int getm_grid_interp_y_f32(int nx, int ny, int nz, const float* source, float* target, int joffset,
                           cudaStream_t stream);
int getm_grid_interp_z_f32(int nx, int ny, int nz1, int nz2, const float* source, float* target,
                           int koffset, cudaStream_t stream);
int getm_grid_interp_xy_f32(int nx1, int ny1, int nx2, int ny2, int nz, const float* source,
                            float* target, int ioffset, int joffset, cudaStream_t stream);
int getm_collect_3d_momentum_sources_f32(int nx, int ny, int nz, int halox, int haloy,
                                         const int* mask, const double* alpha, const double* ho,
                                         const double* hn, const double* dp, const float* cor,
                                         const float* adv, const float* diff, const double* idp,
                                         const double* taus, const double* rr, double dt,
                                         float* ea2, float* ea4, cudaStream_t stream);
int getm_w_momentum_3d_f32(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                           const int* mask, const double* dyu, const double* dxv,
                           const double* iarea, const double* ho, const double* hn,
                           const float* pk, const float* qk, double dt, float* w,
                           cudaStream_t stream);
int getm_shear_frequency_f32(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                             const int* mask, const double* hu, const double* hv, const float* uk,
                             const float* vk, float* SS, cudaStream_t stream);
int getm_reconstruct_transport_change_f32(int nx, int ny, int nz, int imin, int imax, int jmin,
                                          int jmax, float* un, const double* hn, const float* Uo,
                                          double timestep, cudaStream_t stream);
int getm_blumberg_mellor_f32(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                             const int* umask, const int* vmask, const double* idxu,
                             const double* idyv, const double* hu, const double* hv,
                             const double* zf, const float* buoy, float* idpdx, float* idpdy,
                             cudaStream_t stream);
int getm_shchepetkin_mcwilliams_f32(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                                    const int* mask, const int* umask, const int* vmask,
                                    const double* idxu, const double* idyv, const double* h,
                                    const double* z, const double* zc, const float* buoy,
                                    float* idpdx, float* idpdy, double* P_work,
                                    cudaStream_t stream);
int getm_density_buoyancy_f32(int n, const float* salt, const float* temp, const double* p,
                              double* rho, double* buoy, cudaStream_t stream);
/* Squared buoyancy frequency (Density.get_buoyancy_frequency,
 * python/pygetm/density.py:22-60; simulation.py:1200-1204) for the device
 * EOS: at interfaces 1..nz-1 of columns with a non-zero mask,
 * N2 = -g/rho0 (rho(S_k+1, T_k+1, zi) - rho(S_k, T_k, zi)) / dz with zi the
 * mean of the layer-centre depths p and dz the mean thickness; the density
 * difference is formed from the temperature and salinity differences.
 * NN: nz+1 interface levels (surface and bottom left unchanged).  The _f32
 * entry (mixed form) takes float S, T, NN.                                 */
int getm_buoyancy_frequency(int nx, int ny, int nz, const int* mask, const double* h, const double* p,
                            const double* salt, const double* temp, double* NN, cudaStream_t stream);
int getm_buoyancy_frequency_f32(int nx, int ny, int nz, const int* mask, const double* h, const double* p,
                                const float* salt, const float* temp, float* NN, cudaStream_t stream);

/* bottom friction (momentum.F90:79-101, getm_bottom_friction) with the drag
 * coefficient's logarithm and square roots evaluated in float; inputs and
 * outputs stay double.                                                     */
int getm_bottom_friction_mixed(int nx, int ny, const int* mask, const double* u, const double* v,
                               const double* D, double* z0b, const double* z0b_in, double avmmol,
                               double* ru, int iterate, cudaStream_t stream);

/* Shchepetkin-McWilliams internal pressure (internal_pressure.F90:63-217)
 * for the mixed form: same arguments and storage as the FP64 entry point,
 * except that P_work holds nz + 2 planes; the column sums of b dz, the
 * pressure differences and the hydrostatic surface term in FP64 (the sum of
 * the large, nearly cancelling terms), the harmonic-mean slope corrections
 * and the final scaling by the mean thickness and the inverse spacing in
 * float.                                                                   */
int getm_shchepetkin_mcwilliams_mixed(int nx, int ny, int nz, int imin, int imax, int jmin, int jmax,
                                      const int* mask, const int* umask, const int* vmask,
                                      const double* idxu, const double* idyv, const double* h,
                                      const double* z, const double* zc, const double* buoy,
                                      double* idpdx, double* idpdy, double* P_work, cudaStream_t stream);

/* 2D advection of a double field (the depth-averaged momentum of the mixed
 * form) with the same interface as getm_advection_2d (operators.py:52-93)
 * and the same storage, whose increments are evaluated in float in
 * increment form: face deviations are formed from double differences of
 * neighbouring values, the field and the column heights are updated in
 * double.                                                                  */
int getm_advection_2d_mixed(getm_advection* adv, getm_grid* tgrid, getm_grid* ugrid, getm_grid* vgrid,
                            int ufirst, int split, const double* u, const double* v, const double* Ah_u,
                            const double* Ah_v, double timestep, double* D, const double* DU,
                            const double* DV, double* var, cudaStream_t stream);

/* ---- fused sequences of the split-explicit 2D substep ---------------------
 * No single counterpart in the reference: each replaces a sequence of the
 * reference's operations with one launch and, with FP64 arithmetic, gives
 * bitwise the same results as running them one by one (points that a
 * separate interpolation does not write keep their previous values).  All
 * fields are [j][i] with the full extents of their grid (nx, ny of the T
 * grid; X fields nx+1, ny+1).                                              */
/* Simulation.update_depth, 2D part (python/pygetm/simulation.py:1498-1586):
 * elevation2depth of z on T (Dmin -1000), Dclip = max(D, Dmin), z_T_half =
 * (zo + z)/2 and its interpolation to U, V, X (work arrays), depths and
 * alpha there, D_T_half into workT and the UU/VV/UV/VU depth copies.       */
int getm_update_depth_2d(int nx, int ny, double Dmin, double Dcrit, const double* z, const double* zo,
                         const double* HT, const double* HU, const double* HV, const double* HX,
                         const int* mT, const int* mU, const int* mV, const int* mX, double* DT,
                         double* DclipT, double* workT, double* workU, double* DU, double* alphaU,
                         double* workV, double* DV, double* alphaV, double* workX, double* DX,
                         double* DUU, double* DVV, double* DUV, double* DVU, cudaStream_t stream);
/* The same, mixed form: the same depths (minima, maxima and clamps on the
 * integer pipe) and alpha evaluated in float.                              */
int getm_update_depth_2d_mixed(int nx, int ny, double Dmin, double Dcrit, const double* z, const double* zo,
                               const double* HT, const double* HU, const double* HV, const double* HX,
                               const int* mT, const int* mU, const int* mV, const int* mX, double* DT,
                               double* DclipT, double* workT, double* workU, double* DU, double* alphaU,
                               double* workV, double* DV, double* alphaV, double* workX, double* DX,
                               double* DUU, double* DVV, double* DUV, double* DVU, cudaStream_t stream);
/* Momentum._transport_2d_momentum up to its advection calls
 * (python/pygetm/momentum.py:1017-1040): u1 = U/DU, v1 = V/DV, advU = u1,
 * advV = v1, and uua, uva, vua, vva = interpolated transports over the
 * depth of their grid (mixed != 0: these four quotients in float).         */
int getm_momentum_2d_velocities(int nx, int ny, int mixed, const double* U, const double* V,
                                const double* DU, const double* DV, const double* DUU,
                                const double* DUV, const double* DVU, const double* DVV, double* u1,
                                double* v1, double* advU, double* advV, double* uua, double* uva,
                                double* vua, double* vva, cudaStream_t stream);
/* Momentum.bottom_friction (momentum.py:1099-1125): v1 -> U and u1 -> V
 * interpolation into the work arrays, then bottom_friction on both grids
 * (momentum.F90:79-101, no z0b iteration; mixed != 0: float coefficient).  */
int getm_momentum_2d_friction(int nx, int ny, int mixed, const int* mU, const int* mV, const double* u1,
                              const double* v1, const double* DU, const double* DV, const double* z0bU,
                              const double* z0bV, double* workU, double* workV, double* ru, double* rv,
                              cudaStream_t stream);
/* Momentum.coriolis, DEFAULT scheme, 2D (momentum.py:1127-1148): out =
 * (-1 if negate) * f * interp_xy(src, ioffset, joffset).                  */
int getm_coriolis_2d(int nx, int ny, int ioffset, int joffset, const double* src, const double* cor,
                     double* out, int negate, cudaStream_t stream);
/* the same in float arithmetic (mixed form: the transport update reads the
 * term as a float tendency)                                                */
int getm_coriolis_2d_mixed(int nx, int ny, int ioffset, int joffset, const double* src, const double* cor,
                           double* out, int negate, cudaStream_t stream);
/* the same for 3D transports (every layer; nz layers of nx x ny; the _f32
 * entry takes float transports and terms, mixed form)                      */
int getm_coriolis_3d(int nx, int ny, int nz, int ioffset, int joffset, const double* src, const double* cor,
                     double* out, int negate, cudaStream_t stream);
int getm_coriolis_3d_f32(int nx, int ny, int nz, int ioffset, int joffset, const float* src, const double* cor,
                         float* out, int negate, cudaStream_t stream);
/* Momentum.coriolis, ESPELID scheme (momentum.py:1136-1142), 2D (nz = 1,
 * D = water depths) or 3D (D = layer thicknesses): out = (-1 if negate) *
 * f * sqrt(Dout) * interp_xy(src / sqrt(Din)), sqrt(Din) taken as 1 where
 * mask_in == 0; where mask_out == 0 the sqrt(Dout) factor is left out (the
 * reference leaves those points unset).  FP64 arithmetic; the _f32 entry
 * takes float transports and terms.                                        */
int getm_coriolis_espelid(int nx, int ny, int nz, int ioffset, int joffset, const double* src,
                          const double* Din, const int* mask_in, const double* Dout, const int* mask_out,
                          const double* cor, double* out, int negate, cudaStream_t stream);
int getm_coriolis_espelid_f32(int nx, int ny, int nz, int ioffset, int joffset, const float* src,
                              const double* Din, const int* mask_in, const double* Dout, const int* mask_out,
                              const double* cor, float* out, int negate, cudaStream_t stream);
/* advance_2d_transport (momentum.F90:147-189) in the mixed form: tendency
 * summed in float, transport updated in double; same arguments as
 * getm_advance_2d_transport.                                               */
int getm_advance_2d_transport_mixed(int nx, int ny, int halox, int haloy, const int* mask,
                                    const double* alpha, const double* D, const double* dp,
                                    const double* taus, const double* cor, const double* adv,
                                    const double* diff, const double* damp, const double* SA,
                                    const double* SB, const double* SD, const double* SF,
                                    const double* r, double dt, double* U, cudaStream_t stream);
/* _U_cum += U; _V_cum += V (momentum.py:716-718), n points                 */
int getm_accumulate_2d(long long n, const double* U, const double* V, double* Ucum, double* Vcum,
                       cudaStream_t stream);
/* zo = z, then advance_surface_elevation (simulation.py:1468-1486)         */
int getm_surface_elevation_fused(int nx, int ny, int halox, int haloy, const int* mask,
                                 const double* dyu, const double* dxv, const double* iarea, double* z,
                                 double* zo, const double* U, const double* V, const double* fwf,
                                 double dt, cudaStream_t stream);

/* ---- open boundaries (python/pygetm/open_boundaries.py) ------------------
 * Point tables (halo-inclusive T indices i, j; condition type; inward
 * direction di, dj; side 1..4 = W, N, E, S; inflow sign) come from the host
 * collection.  The reference updates its boundaries one after another, so a
 * call covers the contiguous point range [start, stop) of one boundary.    */
/* elevation: ZeroGradient (:338-356), Clamped (:358-375), Flather on
 * elevation or transport (:377-416); result clipped to Dmin - H
 * (simulation.py:580-582, :1252-1257).  z_ext, flow_ext: per point.        */
int getm_open_boundary_elevation(int start, int stop, int nx, const int* i, const int* j,
                                 const int* type, const int* di, const int* dj, const int* side,
                                 const double* inflow_sign, const double* H, const double* Dclip,
                                 const double* U, const double* V, const double* z_ext,
                                 const double* flow_ext, double Dmin, double* z, cudaStream_t stream);
/* tracers (simulation.py:1160-1168): ZeroGradient, Clamped, Sponge with
 * nsponge points (:195-336, fixed relaxation).  vars, bdy: HOST arrays of
 * ntracer (<= 16) device pointers; bdy[t] holds nz x np prescribed values. */
int getm_open_boundary_tracers(int start, int stop, int np, int nx, int ny, int nz, int nsponge,
                               const int* i, const int* j, const int* type, const int* di,
                               const int* dj, const int* mask, int ntracer, double* const* vars,
                               const double* const* bdy, cudaStream_t stream);
int getm_open_boundary_tracers_f32(int start, int stop, int np, int nx, int ny, int nz, int nsponge,
                                   const int* i, const int* j, const int* type, const int* di,
                                   const int* dj, const int* mask, int ntracer, float* const* vars,
                                   const float* const* bdy, cudaStream_t stream);
/* core.Array.mirror (python/pygetm/core.py:723-728): field[tgt] = field[src]
 * for n pairs of flat [j][i] indices, every one of nlev levels of size plane,
 * with every source read before any target is written (a point may be the
 * target of one pair and the source of another); work: device buffer of
 * n * nlev elements.                                                       */
int getm_mirror(int n, const int* src, const int* tgt, int nlev, long long plane, double* field,
                double* work, cudaStream_t stream);
int getm_mirror_f32(int n, const int* src, const int* tgt, int nlev, long long plane, float* field,
                    float* work, cudaStream_t stream);
/* depths at the velocity points just outside boundaries after
 * getm_update_depth_2d: z_T_half.mirror(z_U), elevation2depth, alpha
 * (simulation.py:1545-1552); srcT: boundary T points, tgt: outer points.   */
int getm_open_boundary_depth(int n, const int* srcT, const int* tgt, const double* z, const double* zo,
                             const double* H, const int* mask, double Dmin, double Dcrit, double* work,
                             double* D, double* alpha, cudaStream_t stream);

/* ---- fused 3D momentum array operations ------------------------------------
 * Momentum.advance_3d_transport after the vertical diffusion
 * (python/pygetm/momentum.py:1199-1210) as one sweep per column: tp3d = vel
 * hn, dev = (sum_k tp3d - tp2d) / D, tp3d -= dev hn (the sum in FP64).  The
 * FP64 entry rounds every product and difference as the separate array
 * operations do (the sum runs bottom to top); the _f32 entry (mixed form)
 * forms the products in float.  nx, ny: full extents; tp2d, D, dev: 2D.   */
int getm_transport_3d_finish(int nx, int ny, int nz, const double* vel, const double* hn,
                             const double* tp2d, const double* D, double* tp3d, double* dev,
                             cudaStream_t stream);
int getm_transport_3d_finish_f32(int nx, int ny, int nz, const float* vel, const double* hn,
                                 const double* tp2d, const double* D, float* tp3d, double* dev,
                                 cudaStream_t stream);
/* Column sums of up to four 3D fields into 2D FP64 fields, for the slow
 * terms (momentum.py:989-1012: SxA = sum_k advpk - SxA, ...; simulation.py
 * :1186-1192: SxB = sum_k idpdx): dst = sum_k src, minus the old dst when
 * subtract is non-zero; summed bottom to top in FP64.  Unused pairs are
 * NULL.  nx, ny: full extents.                                              */
int getm_column_sums(int nx, int ny, int nz, int subtract, const double* a3, double* a2,
                     const double* b3, double* b2, const double* c3, double* c2, const double* d3,
                     double* d2, cudaStream_t stream);
int getm_column_sums_f32(int nx, int ny, int nz, int subtract, const float* a3, double* a2,
                         const float* b3, double* b2, const float* c3, double* c2, const float* d3,
                         double* d2, cudaStream_t stream);
/* Inputs of the 3D momentum advection (momentum.py:989-1003) in one launch:
 * uua = interp_x(uk), uva = interp_x(vk), vua = interp_y(uk),
 * vva = interp_y(vk) (offset 0, nz layers), wwu = interp_x(ww),
 * wwv = interp_y(ww) (nz+1 interfaces), advpk = uk, advqk = vk.  Targets
 * keep their values where the interpolation does not write.  nx, ny: full
 * extents (all grids share them).  _f32: float fields (mixed form).       */
int getm_momentum_3d_advection_inputs(int nx, int ny, int nz, const double* uk, const double* vk,
                                      const double* ww, double* uua, double* uva, double* vua, double* vva,
                                      double* wwu, double* wwv, double* advpk, double* advqk,
                                      cudaStream_t stream);
int getm_momentum_3d_advection_inputs_f32(int nx, int ny, int nz, const float* uk, const float* vk,
                                          const float* ww, float* uua, float* uva, float* vua, float* vva,
                                          float* wwu, float* wwv, float* advpk, float* advqk,
                                          cudaStream_t stream);
/* Momentum.update_diagnostics (momentum.py:909-910): uk = pk / hn_U,
 * vk = qk / hn_V over n points (_f32: the division in float).              */
int getm_velocities_3d(long long n, const double* pk, const double* hnu, const double* qk,
                       const double* hnv, double* uk, double* vk, cudaStream_t stream);
int getm_velocities_3d_f32(long long n, const float* pk, const double* hnu, const float* qk,
                           const double* hnv, float* uk, float* vk, cudaStream_t stream);

/* Simulation.update_depth, 3D part (python/pygetm/simulation.py:1588-1630)
 * with Sigma coordinates (vertical_coordinates.py:106-113), in one launch
 * with the arithmetic of the separate array operations: ho = hn (T,
 * U, V); hn = dga Dclip where the mask is non-zero (T, U, V, X);
 * thickness2vertical_coordinates of T, U, V (zc, zf); thickness2center_depth
 * of T into depth (when not NULL); h_T_half = (ho + hn) / 2 and the
 * thicknesses of the UU, VV, UV, VU grids.  dga: nz device values.  nx, ny:
 * full T extents (X fields nx+1 x ny+1).                                    */
typedef struct getm_depth3d_fields {
    const double* dga;
    const int* mask_t; const int* mask_u; const int* mask_v; const int* mask_x;
    const double* Dclip_t; const double* Dclip_u; const double* Dclip_v; const double* Dclip_x;
    const double* H_t; const double* H_u; const double* H_v;
    double* hn_t; double* hn_u; double* hn_v; double* hn_x;
    double* ho_t; double* ho_u; double* ho_v;
    double* zc_t; double* zc_u; double* zc_v; double* zf_t; double* zf_u; double* zf_v;
    double* depth;
    double* h_T_half; double* hn_uu; double* hn_vv; double* hn_uv; double* hn_vu;
} getm_depth3d_fields;

int getm_update_depth_3d(const getm_depth3d_fields* f, int nx, int ny, int nz, cudaStream_t stream);

/* ---- one 2D substep as one launch -----------------------------------------
 * Replaces, for a substep of python/pygetm/simulation.py:291-325
 * (Simulation.advance) that is not followed by a 3D step, the sequence
 * simulation.py:1033-1039 (momentum.advance_depth_integrated, momentum.py
 * :644-718, and advance_surface_elevation, :1468-1486) and :1138-1304 with
 * update_3d false: update_depth (2D part, :1498-1586), the momentum
 * diagnostics with skip_coriolis (momentum.py:720-758, :1017-1125) without
 * horizontal diffusion and without the z0b iteration, fwf = pe, the surface
 * pressure gradient and the wind-stress interpolation; plus time += dt.
 * Closed domains (no open boundaries), DEFAULT Coriolis scheme, FULL 2D
 * advection split.  Results are bitwise those of the separate operations.
 * mixed: 0 FP64 form, 1 mixed form (float tendencies, increment-form 2D
 * advection; getm_advance_2d_transport_mixed, getm_advection_2d_mixed).
 * ufirst: momentum order of this substep (U then V); accumulate: add U, V to
 * Ucum, Vcum (3D runs); friction: bottom friction (ru, rv).  uadv/vadv: the
 * momentum advection handles with their grids (T = U resp. V grid) and their
 * u-first flags.  sync: 4 words, zero before the first call; sync[2] != 0
 * after a call means a grid barrier gave up (the call did not complete and
 * every later call returns at once until the word is cleared).  All fields
 * are [j][i] with the full extents nx, ny (X fields nx+1, ny+1).            */
typedef struct getm_split2d_fields {
    /* T grid */
    const int* mask_t; const double* H_t; const double* iarea_t;
    double* z; double* zo; double* D_t; double* Dclip_t; double* work_t;
    double* fwf; const double* pe; const double* sp; const double* taux; const double* tauy;
    /* U grid and the U momentum equation */
    const int* mask_u; const double* H_u; const double* dy_u; const double* idx_u; const double* cor_u;
    const double* z0b_u; double* D_u; double* alpha_u; double* work_u;
    double* U; double* dpdx; double* tausx; double* corU; double* advU; const double* diffU;
    const double* dampU; const double* SxA; const double* SxB; const double* SxD; const double* SxF;
    double* ru; double* u1; double* Ucum; double* advD_u; double* uua; double* uva;
    /* V grid and the V momentum equation */
    const int* mask_v; const double* H_v; const double* dx_v; const double* idy_v; const double* cor_v;
    const double* z0b_v; double* D_v; double* alpha_v; double* work_v;
    double* V; double* dpdy; double* tausy; double* corV; double* advV; const double* diffV;
    const double* dampV; const double* SyA; const double* SyB; const double* SyD; const double* SyF;
    double* rv; double* v1; double* Vcum; double* advD_v; double* vua; double* vva;
    /* X grid and the depths of the advection velocity grids */
    const int* mask_x; const double* H_x; double* D_x; double* work_x;
    double* D_uu; double* D_uv; double* D_vu; double* D_vv;
    double* time;          /* may be NULL */
    unsigned int* sync;
} getm_split2d_fields;

int getm_split2d_substep(const getm_split2d_fields* f, int nx, int ny, int halox, int haloy, int mixed,
                         int ufirst, int accumulate, int friction, double timestep, double Dmin, double Dcrit,
                         getm_advection* uadv, getm_grid* ugrid, getm_grid* uugrid, getm_grid* uvgrid,
                         int uadv_ufirst, getm_advection* vadv, getm_grid* vgrid, getm_grid* vugrid,
                         getm_grid* vvgrid, int vadv_ufirst, cudaStream_t stream);

/* ---- turbulence closure -----------------------------------------------
 * Replaces the GOTM call of python/pygetm/vertical_mixing.py:150-188
 * (VerticalMixing GOTM.advance: tke, eps, L, num, nuh at the interfaces
 * from ustar_s, ustar_b, z0s, z0b, NN and SS, once per 3D step).  GOTM is
 * external to the reference; this is the buoyancy-extended k-epsilon model
 * of Rodi (1987) with constant stability functions (num = cm0^4 k^2/eps,
 * nuh = num/prandtl), log-law Dirichlet values at the bottom and surface
 * interfaces (k = ustar^2/cm0^2, eps = cm0^3 k^1.5/(kappa z0)), implicit
 * diffusion of k (num/sig_k) and eps (num/sig_e) with Patankar-linearised
 * sources, k >= k_min, eps >= eps_min and the Galperin limit L <= galp
 * sqrt(2k/NN) where NN > 0.  FP64; one thread per water column (mask == 1,
 * interior); fields are nz + 1 interface planes of nx x ny (halos
 * included), h has nz layers; work: 2 (nz + 1) nx ny doubles.              */
typedef struct getm_keps_params {
    double cm0, kappa, sig_k, sig_e, c1, c2, c3_minus, c3_plus, galp, prandtl, k_min, eps_min;
} getm_keps_params;
int getm_keps_default_params(getm_keps_params* p);
int getm_keps_advance(int nx, int ny, int nz, int halox, int haloy, const getm_keps_params* params,
                      double timestep, const int* mask, const double* h, const double* ustar_s,
                      const double* ustar_b, const double* z0s, const double* z0b, const double* NN,
                      const double* SS, double* tke, double* eps, double* L, double* num, double* nuh,
                      double* work, cudaStream_t stream);
/* the mixed form: NN, SS, num and nuh in float (k, eps, L and the
 * arithmetic stay FP64)                                                     */
int getm_keps_advance_f32(int nx, int ny, int nz, int halox, int haloy, const getm_keps_params* params,
                          double timestep, const int* mask, const double* h, const double* ustar_s,
                          const double* ustar_b, const double* z0s, const double* z0b, const float* NN,
                          const float* SS, double* tke, double* eps, double* L, float* num, float* nuh,
                          double* work, cudaStream_t stream);

/* ---- substeps of many domains in one launch ------------------------------
 * No single counterpart in the reference, which advances each domain in its
 * own process: for an ensemble of independent domains (each one
 * Simulation.advance substep sequence, python/pygetm/simulation.py:291-325),
 * the substeps that are not followed by a 3D step run for all members
 * together, one cooperative launch per substep index k, with the operations
 * and results of getm_split2d_substep per member.
 *   create(nmember, mixed): a table for nmember domains of one form;
 *   set(member, nsub, split, <getm_split2d_substep's arguments>): member's
 *     fields at the start of a round of `split` substeps, nsub of which (the
 *     ones without 3D step, split - 1 in a split-explicit run) run here; its
 *     transport order `ufirst` is the order of its first substep in a round
 *     of even parity;
 *   upload(b): builds the device table (cudaMalloc and synchronous copies:
 *     call before any stream capture; set() is closed afterwards);
 *   launch(b, k, round_parity, sync): substep k of the round for every member
 *     with nsub > k (round_parity: the round's index mod 2; a member's order
 *     then is its recorded order flipped k + round_parity * split times);
 *     sync: 4 zeroed barrier words owned by the caller, as for
 *     getm_split2d_substep (its bounded waits and error word).
 *   participants(b, k, count): members that take part in launch k.          */
typedef struct getm_substep_batch getm_substep_batch;
int getm_substep_batch_create(int nmember, int mixed, getm_substep_batch** out);
int getm_substep_batch_set(getm_substep_batch* b, int member, int nsub, int split, const getm_split2d_fields* f,
                           int nx, int ny, int halox, int haloy, int ufirst, int accumulate, int friction,
                           double timestep, double Dmin, double Dcrit, getm_advection* uadv, getm_grid* ugrid,
                           getm_grid* uugrid, getm_grid* uvgrid, int uadv_ufirst, getm_advection* vadv,
                           getm_grid* vgrid, getm_grid* vugrid, getm_grid* vvgrid, int vadv_ufirst);
int getm_substep_batch_upload(getm_substep_batch* b);
int getm_substep_batch_participants(const getm_substep_batch* b, int k, int* count);
int getm_substep_batch_launch(getm_substep_batch* b, int k, int round_parity, unsigned int* sync,
                              cudaStream_t stream);
int getm_substep_batch_finalize(getm_substep_batch* b);

/* ---- domain totals (compensated budget sums) -----------------------------
 * Replaces python/pygetm/simulation.py:1409-1444 (Simulation.totals: total
 * volume = sum of D*area, tracer total = sum of c*area*hn over unmasked
 * interior points) and the Array.global_sum it calls
 * (python/pygetm/core.py:820-839).  Sums are double-double (error-free
 * transformations) in a fixed reduction order: correctly rounded to a few
 * ulps and bitwise reproducible.  nx_/ny_: full extents; nx/ny: interior
 * extents starting at (halox, haloy).  tracers: HOST array of ntracer
 * device pointers (nz layers each).  work: device buffer of
 * 2 * GETM_TOTALS_BLOCKS * (1 + ntracer) doubles.  out: device array of
 * 1 + ntracer doubles (volume, then each tracer).                          */
int getm_domain_totals(int nx_, int ny_, int nz, int halox, int haloy, int nx, int ny,
                       const int* mask, const double* area, const double* D, const double* hn,
                       int ntracer, const double* const* tracers, double* work, double* out,
                       cudaStream_t stream);
int getm_domain_totals_f32(int nx_, int ny_, int nz, int halox, int haloy, int nx, int ny,
                           const int* mask, const double* area, const double* D, const double* hn,
                           int ntracer, const float* const* tracers, double* work, double* out,
                           cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* GETM_GB300_H */
