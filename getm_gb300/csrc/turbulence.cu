// Two-equation (k-epsilon) turbulence closure for sm_103a: the turbulent
// viscosity num and diffusivity nuh at the layer interfaces.
//
// pygetm takes num and nuh from GOTM through pygotm
// (python/pygetm/vertical_mixing.py:60-188, advanced once per 3D step at
// python/pygetm/simulation.py:1107-1115 with ustar_s, ustar_b, z0s, z0b, NN and
// SS).  GOTM is an external package that the reference does not vendor, so
// this is not its code: it is the buoyancy-extended k-epsilon model of Rodi
// (1987, J. Geophys. Res. 92, "Examples of calculation methods for flow and
// mixing in stratified fluids") with constant stability functions, the
// standard model constants (Launder and Spalding 1974), log-law (Dirichlet)
// boundary values for k and epsilon at the bottom and surface interfaces,
// the length-scale limitation of Galperin et al. (1988) in stable
// stratification, and the source-term linearisation of Patankar (1980)
// that keeps k and epsilon positive in the implicit update:
//
//   dk/dt   = d/dz (num/sk dk/dz) + P + B - eps
//   deps/dt = d/dz (num/se deps/dz) + eps/k (c1 P + c3 B - c2 eps)
//   P = num SS, B = -nuh NN, num = cmu k^2/eps, nuh = num / Prt
//
// One thread per water column (32 columns of a warp are adjacent at every
// level, so each level's loads are coalesced); both equations are solved
// implicitly in time over the interfaces 1..nz-1 with a Thomas sweep whose
// elimination coefficients live in a [level][column] workspace.
#include "getm_common.cuh"

namespace {

// R: type of NN, SS, num and nuh (float in the mixed form); k, epsilon and
// L are FP64 in both forms, and so is the arithmetic.
template <typename R>
struct KepsArgs {
    int nx, ny, nz;
    long long plane;
    int ilo, ihi, jlo, jhi;
    const int* mask;
    const double* h;  // layer thicknesses, nz layers
    const double *ustar_s, *ustar_b, *z0s, *z0b;
    const R *NN, *SS;  // nz + 1 interfaces
    double *tke, *eps, *L;
    R *num, *nuh;
    double* work;  // 2 (nz + 1) planes
    double dt;
    getm_keps_params p;
};

// log-law boundary values at the interface at distance z0 from the wall
__device__ __forceinline__ void keps_wall(const getm_keps_params& p, double ustar, double z0, double& k, double& e)
{
    const double cm0 = p.cm0;
    k = fmax(ustar * ustar / (cm0 * cm0), p.k_min);
    e = fmax(cm0 * cm0 * cm0 * k * sqrt(k) / (p.kappa * z0), p.eps_min);
}

// One implicit diffusion-source equation over interfaces 1..nz-1 of column
// c: dz_i (x_i' - x_i) / dt = flux differences + dz_i (Q_i + S_i x_i'),
// diffusivities K at the layers (between interfaces), Dirichlet values x0,
// xn at interfaces 0 and nz.  Q and S come from src(i, Q, S).
template <typename R, typename Src, typename Diff>
__device__ __forceinline__ void keps_solve(const KepsArgs<R>& a, long long c, double* x, double x0, double xn,
                                           Src src, Diff kdiff)
{
    const long long P = a.plane;
    const int nz = a.nz;
    double* cp = a.work + c;
    double* dp = a.work + (long long)(nz + 1) * P + c;
    double cprev = 0.0, dprev = x0;  // interface 0 is fixed
    double hb = a.h[c];              // layer below interface i
    double Kb = kdiff(0);
    for (int i = 1; i < nz; i++) {
        const double ht = a.h[c + (long long)i * P];  // layer above interface i
        const double Kt = kdiff(i);
        const double dz = 0.5 * (hb + ht);
        double Q, S;
        src(i, Q, S);
        const double lo = -a.dt * Kb / hb;
        const double up = -a.dt * Kt / ht;
        const double b = dz - lo - up - a.dt * dz * S;
        double d = dz * (x[c + (long long)i * P] + a.dt * Q);
        if (i == nz - 1) d -= up * xn;
        const double den = b - lo * cprev;
        cprev = up / den;
        dprev = (d - lo * dprev) / den;
        cp[(long long)i * P] = cprev;
        dp[(long long)i * P] = dprev;
        hb = ht;
        Kb = Kt;
    }
    double xv = xn;
    for (int i = nz - 1; i >= 1; i--) {
        xv = dp[(long long)i * P] - cp[(long long)i * P] * xv;
        x[c + (long long)i * P] = xv;
    }
    x[c] = x0;
    x[c + (long long)nz * P] = xn;
}

template <typename R>
__global__ void __launch_bounds__(128) keps_kernel(KepsArgs<R> a)
{
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < a.ilo || i > a.ihi || j < a.jlo || j > a.jhi) return;
    const long long c = (long long)j * a.nx + i;
    if (a.mask[c] != 1) return;
    const getm_keps_params& p = a.p;
    const long long P = a.plane;
    const int nz = a.nz;
    const double cmu = p.cm0 * p.cm0 * p.cm0 * p.cm0;
    const double cde = p.cm0 * p.cm0 * p.cm0;
    double kb, eb, ks, es;
    keps_wall(p, a.ustar_b[c], a.z0b[c], kb, eb);
    keps_wall(p, a.ustar_s[c], a.z0s[c], ks, es);

    // turbulent kinetic energy (old epsilon and diffusivities in the sources)
    auto kdiff_k = [&](int l) {
        return 0.5 * ((double)a.num[c + (long long)l * P] + (double)a.num[c + (long long)(l + 1) * P]) / p.sig_k;
    };
    auto src_k = [&](int l, double& Q, double& S) {
        const long long q = c + (long long)l * P;
        const double prod = (double)a.num[q] * (double)a.SS[q], buoy = -(double)a.nuh[q] * (double)a.NN[q];
        const double k = a.tke[q], e = a.eps[q];
        if (prod + buoy > 0.0) { Q = prod + buoy; S = -e / k; }
        else { Q = prod; S = -(e - buoy) / k; }
    };
    // (the forward sweep reads every old value before the back substitution
    // overwrites them, so the update is in place)
    keps_solve(a, c, a.tke, kb, ks, src_k, kdiff_k);
    for (int l = 1; l < nz; l++) {
        const long long q = c + (long long)l * P;
        a.tke[q] = fmax(a.tke[q], p.k_min);
    }

    // dissipation rate (sources from the new k and the old epsilon)
    auto kdiff_e = [&](int l) {
        return 0.5 * ((double)a.num[c + (long long)l * P] + (double)a.num[c + (long long)(l + 1) * P]) / p.sig_e;
    };
    auto src_e = [&](int l, double& Q, double& S) {
        const long long q = c + (long long)l * P;
        const double prod = (double)a.num[q] * (double)a.SS[q], buoy = -(double)a.nuh[q] * (double)a.NN[q];
        const double r = a.eps[q] / a.tke[q];
        const double c3 = buoy > 0.0 ? p.c3_plus : p.c3_minus;
        Q = r * (p.c1 * prod + c3 * buoy);
        S = -p.c2 * r;
    };
    keps_solve(a, c, a.eps, eb, es, src_e, kdiff_e);

    // limits, length scale, viscosity and diffusivity at every interface
    for (int l = 0; l <= nz; l++) {
        const long long q = c + (long long)l * P;
        const double k = a.tke[q];
        double e = fmax(a.eps[q], p.eps_min);
        const double N2 = (double)a.NN[q];
        if (l > 0 && l < nz && N2 > 0.0) {  // Galperin: L <= galp sqrt(2 k / N2)
            const double lmax = p.galp * sqrt(2.0 * k / N2);
            e = fmax(e, cde * k * sqrt(k) / lmax);
        }
        a.eps[q] = e;
        a.L[q] = cde * k * sqrt(k) / e;
        const double nu = cmu * k * k / e;
        a.num[q] = (R)nu;
        a.nuh[q] = (R)(nu / p.prandtl);
    }
}

}  // namespace

extern "C" int getm_keps_default_params(getm_keps_params* p)
{
    if (!p) return GETM_ERR_ARG;
    p->cm0 = 0.5477;
    p->kappa = 0.4;
    p->sig_k = 1.0;
    p->sig_e = 1.3;
    p->c1 = 1.44;
    p->c2 = 1.92;
    p->c3_minus = -0.4;
    p->c3_plus = 1.0;
    p->galp = 0.53;
    p->prandtl = 1.0;
    p->k_min = 1e-10;
    p->eps_min = 1e-12;
    return GETM_OK;
}

template <typename R>
static int keps_impl(int nx, int ny, int nz, int halox, int haloy, const getm_keps_params* params, double timestep,
                     const int* mask, const double* h, const double* ustar_s, const double* ustar_b,
                     const double* z0s, const double* z0b, const R* NN, const R* SS, double* tke, double* eps,
                     double* L, R* num, R* nuh, double* work, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 2 || halox < 0 || haloy < 0 || !params || !(timestep > 0.0)) return GETM_ERR_ARG;
    const void* ptrs[] = {mask, h, ustar_s, ustar_b, z0s, z0b, NN, SS, tke, eps, L, num, nuh, work};
    for (const void* q : ptrs)
        if (!q) return GETM_ERR_ARG;
    KepsArgs<R> a;
    a.nx = nx; a.ny = ny; a.nz = nz; a.plane = (long long)nx * ny;
    a.ilo = halox; a.ihi = nx - halox - 1; a.jlo = haloy; a.jhi = ny - haloy - 1;
    a.mask = mask; a.h = h; a.ustar_s = ustar_s; a.ustar_b = ustar_b; a.z0s = z0s; a.z0b = z0b;
    a.NN = NN; a.SS = SS; a.tke = tke; a.eps = eps; a.L = L; a.num = num; a.nuh = nuh; a.work = work;
    a.dt = timestep;
    a.p = *params;
    const dim3 grid(getm_div_up(nx, 32), getm_div_up(ny, 4)), block(32, 4);
    keps_kernel<R><<<grid, block, 0, stream>>>(a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_keps_advance(int nx, int ny, int nz, int halox, int haloy, const getm_keps_params* params,
                                 double timestep, const int* mask, const double* h, const double* ustar_s,
                                 const double* ustar_b, const double* z0s, const double* z0b, const double* NN,
                                 const double* SS, double* tke, double* eps, double* L, double* num, double* nuh,
                                 double* work, cudaStream_t stream)
{
    return keps_impl<double>(nx, ny, nz, halox, haloy, params, timestep, mask, h, ustar_s, ustar_b, z0s, z0b, NN, SS,
                             tke, eps, L, num, nuh, work, stream);
}

extern "C" int getm_keps_advance_f32(int nx, int ny, int nz, int halox, int haloy, const getm_keps_params* params,
                                     double timestep, const int* mask, const double* h, const double* ustar_s,
                                     const double* ustar_b, const double* z0s, const double* z0b, const float* NN,
                                     const float* SS, double* tke, double* eps, double* L, float* num, float* nuh,
                                     double* work, cudaStream_t stream)
{
    return keps_impl<float>(nx, ny, nz, halox, haloy, params, timestep, mask, h, ustar_s, ustar_b, z0s, z0b, NN, SS,
                            tke, eps, L, num, nuh, work, stream);
}
