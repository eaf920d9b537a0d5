// Implicit (Crank-Nicolson) vertical diffusion for sm_103a.
//
// Reference: src/operators/diffusion.F90 (prepare :135-204, apply :206-314)
// reached through python/src/wrapper.F90:127-186 and
// python/pygetm/operators.py:218-230 (VerticalDiffusion).
//
// GB300 design: one thread per water column.  The C layout [k][j][i] puts the
// 32 columns of a warp next to each other at every level, so each per-level
// load/store of the sweep is a fully coalesced 256-byte transaction.  The
// tridiagonal matrix is never stored: its coefficients are formed on the fly
// from nuh, ho, hn and var while sweeping down from the surface (the Thomas
// forward elimination of diffusion.F90:285-292), keeping only the two
// elimination coefficients per level for the back substitution (:304-307),
// in shared memory or in a caller-provided global workspace.  prepare+apply
// are fused (traffic per field: read nuh, ho, hn, var [+ea2, ea4], write
// var).  The mixed form's solve (vd_inc_kernel) takes fields in pairs and
// issues each level's loads one level ahead.  A warp-per-column PCR solve would
// cost O(nz log nz) FP64 divides per column instead of O(nz); GB300's FP64
// rate makes the serial Thomas sweep the faster choice for the FP64 form.
// For domains with few columns the mixed form can instead split each column
// into four segments, one warp each (vd_seg_kernel, the partition method).
#include <stdlib.h>
#include <string.h>

#include "getm_common.cuh"

#define VD_MAX_BATCH 32

struct getm_vertical_diffusion {
    getm_grid* tgrid;
    size_t n3;
    double* auxo;   // prepare -> apply work arrays (diffusion.F90:88)
    double* auxn;
};

// T: type of nuh and of the solve (double: FP64 form; float: mixed form);
// S: storage type of the diffused fields (T unless given; double with a
// float solve: the mixed form with FP64 tracer storage, increment form).
// Layer thicknesses are double in every form.
template <typename T, typename S = T>
struct VDArgs {
    int nx_, ny_, nz;
    long long plane;
    const int* mask;
    const T* nuh;          // nz+1 interface levels
    const double* ho;
    const double* hn;
    const double* auxo;    // FP64 form, when prepared separately (else NULL)
    const double* auxn;
    double dt, cnpar;
    int ntracer;
    double molecular[VD_MAX_BATCH];
    S* var[VD_MAX_BATCH];
    const T* ea2[VD_MAX_BATCH];
    const T* ea4[VD_MAX_BATCH];
    T* work;               // NULL, or 2 nz plane elements: elimination coefficients in global memory
};

// A layer thickness in the solve's type (the mixed form converts on the
// integer pipe, see getm_d2f_approx).
template <typename T>
__device__ __forceinline__ T vd_h(double h)
{
    if constexpr (getm_increment_form<T>) return getm_d2f_approx(h);
    else return h;
}

// Coupling coefficients of the interface above C level k (between levels k and
// k+1): diffusion.F90:166-168 with Fortran k = C k + 1.
template <typename T>
__device__ __forceinline__ void vd_aux(const VDArgs<T>& a, long long c, int k, double mol, T& auxo, T& auxn)
{
    const long long P = a.plane;
    if (a.auxo) {
        auxo = (T)a.auxo[c + k * P];
        auxn = (T)a.auxn[c + k * P];
        return;
    }
    T x = (T)(2.0 * a.dt) * (a.nuh[c + (k + 1) * P] + (T)mol);
    auxo = (T)(1.0 - a.cnpar) * x / (vd_h<T>(a.ho[c + (k + 1) * P]) + vd_h<T>(a.ho[c + k * P]));
    auxn = (T)a.cnpar * x / (vd_h<T>(a.hn[c + (k + 1) * P]) + vd_h<T>(a.hn[c + k * P]));
}

// Increment form: (ho - hn) of one layer as float, exact-difference first;
// zero without FP64 work when the solve uses one thickness (ho == hn).
__device__ __forceinline__ float vd_dh(const double* ho, const double* hn, long long q)
{
    return ho == hn ? 0.f : getm_d2f_approx(ho[q] - hn[q]);
}

// Thread per column; dynamic shared memory holds ru/qu (and, in the
// increment form, the old values): vd_smem_arrays<T> * nz * blockDim values.
//
// Increment form (float): with x the old values and A x_new = a4 the
// reference system, the kernel solves A dx = a4 - A x, whose right-hand side
// reduces to differences that float32 holds exactly or nearly so:
//   r_k = x_k (ho_k - hn_k) + (x_{k+1} - x_k)(auxo + auxn)_{k+1/2}
//         + (x_{k-1} - x_k)(auxo + auxn)_{k-1/2} + ea4_k + ea2_k x_k
// and writes x + dx.
template <typename T>
constexpr int vd_smem_arrays = getm_increment_form<T> ? 3 : 2;

// GW: the elimination coefficients ru, qu live in a.work ([k][j][i], so every
// level is again one coalesced access) instead of shared memory, which then
// no longer limits the number of resident columns; the increment form
// re-reads the old values from var during the back substitution (var[k] is
// overwritten only after it is read).
template <typename T, bool GW>
__global__ void __launch_bounds__(128, getm_increment_form<T> ? 8 : 1) vd_column_kernel(VDArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char vd_smem[];
    constexpr bool inc = getm_increment_form<T>;
    const int tid = threadIdx.x;
    const int nthreads = blockDim.x;
    const int i = blockIdx.x * blockDim.x + tid;
    const int j = blockIdx.y;
    if (i >= a.nx_) return;
    const long long c = (long long)j * a.nx_ + i;
    const long long P = a.plane;
    const int nz = a.nz;
    if (nz == 1) {  // diffusion.F90:224-231: every point, mask not consulted
        for (int t = 0; t < a.ntracer; t++) {
            T x = a.var[t][c];
            T a2 = vd_h<T>(a.hn[c]);
            if (a.ea2[t]) a2 = a2 - a.ea2[t][c];
            if constexpr (inc) {
                T r = x * vd_dh(a.ho, a.hn, c);
                if (a.ea4[t]) r = r + a.ea4[t][c];
                if (a.ea2[t]) r = r + a.ea2[t][c] * x;
                a.var[t][c] = x + r / a2;
            } else {
                T a4 = vd_h<T>(a.ho[c]) * x;
                if (a.ea4[t]) a4 = a4 + a.ea4[t][c];
                a.var[t][c] = a4 / a2;
            }
        }
        return;
    }
    if (a.mask[c] != 1) return;
    // ru[k * rs], qu[k * rs] (and xo[k * rs], increment form in shared memory)
    T* ru;
    T* qu;
    T* xo;
    long long rs;
    if constexpr (GW) {
        ru = a.work + c;
        qu = ru + P * nz;
        xo = a.var[0] + c;  // not used: old values are re-read from var
        rs = P;
    } else {
        ru = (T*)vd_smem + tid;
        qu = ru + (size_t)nz * nthreads;
        xo = qu + (size_t)nz * nthreads;
        rs = nthreads;
    }
    for (int t = 0; t < a.ntracer; t++) {
        T* __restrict__ var = a.var[t];
        const T* ea2 = a.ea2[t];
        const T* ea4 = a.ea4[t];
        const double mol = a.molecular[t];
        // surface layer (C level nz-1), diffusion.F90:238-245
        int k = nz - 1;
        T aob, anb;                             // aux of the interface below level k
        vd_aux(a, c, k - 1, mol, aob, anb);
        T vk = var[c + k * P];
        T vkm1 = var[c + (k - 1) * P];
        T a1 = -anb;
        T a2 = vd_h<T>(a.hn[c + k * P]) + anb;
        T a4;
        if constexpr (inc) {
            if constexpr (!GW) xo[k * rs] = vk;
            a4 = vk * vd_dh(a.ho, a.hn, c + k * P) + (vkm1 - vk) * (aob + anb);
            if (ea2) a4 = a4 + ea2[c + k * P] * vk;
        } else {
            a4 = vk * (T)a.ho[c + k * P] + (vkm1 - vk) * aob;
        }
        if (ea2) a2 = a2 - ea2[c + k * P];
        if (ea4) a4 = a4 + ea4[c + k * P];
        T rk = a1 / a2;
        T qk = a4 / a2;
        ru[k * rs] = rk;
        qu[k * rs] = qk;
        // inner layers, diffusion.F90:247-258 and elimination :287-290
        T aoa = aob, ana = anb;                 // interface above level k-1
        T vkp1 = vk;
        vk = vkm1;
        for (k = nz - 2; k >= 1; k--) {
            vd_aux(a, c, k - 1, mol, aob, anb);
            vkm1 = var[c + (k - 1) * P];
            T a3 = -ana;
            a1 = -anb;
            a2 = vd_h<T>(a.hn[c + k * P]) + ana + anb;
            if constexpr (inc) {
                if constexpr (!GW) xo[k * rs] = vk;
                a4 = vk * vd_dh(a.ho, a.hn, c + k * P) + (vkp1 - vk) * (aoa + ana) +
                     (vkm1 - vk) * (aob + anb);
                if (ea2) a4 = a4 + ea2[c + k * P] * vk;
            } else {
                a4 = vk * (T)a.ho[c + k * P] + (vkp1 - vk) * aoa + (vkm1 - vk) * aob;
            }
            if (ea2) a2 = a2 - ea2[c + k * P];
            if (ea4) a4 = a4 + ea4[c + k * P];
            T den = a2 - a3 * rk;
            rk = a1 / den;
            qk = (a4 - a3 * qk) / den;
            ru[k * rs] = rk;
            qu[k * rs] = qk;
            aoa = aob; ana = anb;
            vkp1 = vk; vk = vkm1;
        }
        // bottom layer, diffusion.F90:260-267 and :291-292
        {
            T a3 = -ana;
            a2 = vd_h<T>(a.hn[c]) + ana;
            if constexpr (inc) {
                a4 = vk * vd_dh(a.ho, a.hn, c) + (vkp1 - vk) * (aoa + ana);
                if (ea2) a4 = a4 + ea2[c] * vk;
            } else {
                a4 = vk * (T)a.ho[c] + (vkp1 - vk) * aoa;
            }
            if (ea2) a2 = a2 - ea2[c];
            if (ea4) a4 = a4 + ea4[c];
            T q0 = (a4 - a3 * qk) / (a2 - a3 * rk);
            // back substitution :304-307
            T vprev = q0;
            if constexpr (inc) {
                var[c] = vk + q0;
                for (k = 1; k < nz; k++) {
                    vprev = qu[k * rs] - ru[k * rs] * vprev;
                    const T x_old = GW ? var[c + k * P] : xo[k * rs];
                    var[c + k * P] = x_old + vprev;
                }
            } else {
                var[c] = q0;
                for (k = 1; k < nz; k++) {
                    vprev = qu[k * rs] - ru[k * rs] * vprev;
                    var[c + k * P] = vprev;
                }
            }
        }
    }
}

// Increment form with the elimination coefficients in global memory (the
// mixed form's column solve): the same arithmetic as vd_column_kernel<float,
// true>, restructured for memory-level parallelism.  The loads of the
// forward elimination do not depend on the elimination itself, so the
// operands of the next level (thicknesses, nuh, field values, sources) are
// issued one level ahead of the arithmetic, and those of the back
// substitution likewise; NT fields share the thickness and nuh loads and
// sweep together (work: 2 nz planes per field of a group).  SRC: whether a
// field of the group has ea2 or ea4 (without, no registers are spent on
// them).
template <int NT, bool SRC, typename S>
__device__ __forceinline__ void vd_inc_sweep(const VDArgs<float, S>& a, long long c, int t0)
{
    const long long P = a.plane;
    const int nz = a.nz;
    const double* __restrict__ ho = a.ho + c;
    const double* __restrict__ hn = a.hn + c;
    const float* __restrict__ nuh = a.nuh + c;
    const bool one_h = a.ho == a.hn;
    const float co = (float)(1.0 - a.cnpar), cn = (float)a.cnpar, dt2 = (float)(2.0 * a.dt);
    S* v[NT];
    const float* e2[NT];
    const float* e4[NT];
    float* ru[NT];
    float* qu[NT];
    float mol[NT];
#pragma unroll
    for (int t = 0; t < NT; t++) {
        v[t] = a.var[t0 + t] + c;
        e2[t] = SRC && a.ea2[t0 + t] ? a.ea2[t0 + t] + c : nullptr;
        e4[t] = SRC && a.ea4[t0 + t] ? a.ea4[t0 + t] + c : nullptr;
        ru[t] = a.work + c + (long long)(2 * t) * nz * P;
        qu[t] = ru[t] + (long long)nz * P;
        mol[t] = (float)a.molecular[t0 + t];
    }
    // level k operands (current) and the raw loads of level k-1 (next)
    int k = nz - 1;
    double ho_c = ho[k * P], hn_c = hn[k * P];
    double ho_n = ho[(k - 1) * P], hn_n = hn[(k - 1) * P];
    float nuh_c = nuh[k * P];  // interface below level k
    S vk[NT], vn[NT];
    float e2c[NT], e4c[NT];
#pragma unroll
    for (int t = 0; t < NT; t++) {
        vk[t] = v[t][k * P];
        vn[t] = v[t][(k - 1) * P];
        e2c[t] = SRC && e2[t] ? e2[t][k * P] : 0.f;
        e4c[t] = SRC && e4[t] ? e4[t][k * P] : 0.f;
    }
    float hoF = vd_h<float>(ho_c), hnF = vd_h<float>(hn_c);
    float dh = one_h ? 0.f : getm_d2f_approx(ho_c - hn_c);
    float rk[NT], qk[NT], aoa[NT], ana[NT], dprev[NT];
    // surface layer (diffusion.F90:238-245) and the inner layers
    // (:247-258, elimination :287-290)
    for (; k >= 1; k--) {
        // next level's raw operands, one level ahead
        const int kn = k - 1;
        double ho_nn = 0.0, hn_nn = 0.0;
        float nuh_n = 0.f, e2n[NT], e4n[NT];
        S vnn[NT];
        if (kn >= 1) {
            ho_nn = ho[(kn - 1) * P];
            hn_nn = hn[(kn - 1) * P];
        }
        nuh_n = nuh[kn * P];
#pragma unroll
        for (int t = 0; t < NT; t++) {
            vnn[t] = kn >= 1 ? v[t][(kn - 1) * P] : S(0);
            e2n[t] = SRC && e2[t] ? e2[t][kn * P] : 0.f;
            e4n[t] = SRC && e4[t] ? e4[t][kn * P] : 0.f;
        }
        // interface below level k (vd_aux with C level k-1)
        const float hoFn = vd_h<float>(ho_n), hnFn = vd_h<float>(hn_n);
        const float so = hoF + hoFn, sn = hnF + hnFn;
#pragma unroll
        for (int t = 0; t < NT; t++) {
            const float x = dt2 * (nuh_c + mol[t]);
            const float aob = co * x / so;
            const float anb = cn * x / sn;
            const float a1 = -anb;
            // differences of neighbouring values in the storage type, then
            // narrowed (exact for float storage); the difference to the
            // level above is minus the level above's difference to this one
            const float xk = inc_f<S>(vk[t]);
            const float ddn = inc_f<S>(vn[t] - vk[t]);
            float a2, a4;
            if (k == nz - 1) {
                a2 = hnF + anb;
                a4 = xk * dh + ddn * (aob + anb);
            } else {
                a2 = hnF + ana[t] + anb;
                a4 = xk * dh + (-dprev[t]) * (aoa[t] + ana[t]) + ddn * (aob + anb);
            }
            dprev[t] = ddn;
            if (SRC && e2[t]) a4 = a4 + e2c[t] * xk;
            if (SRC && e2[t]) a2 = a2 - e2c[t];
            if (SRC && e4[t]) a4 = a4 + e4c[t];
            if (k == nz - 1) {
                rk[t] = a1 / a2;
                qk[t] = a4 / a2;
            } else {
                const float a3 = -ana[t];
                const float den = a2 - a3 * rk[t];
                rk[t] = a1 / den;
                qk[t] = (a4 - a3 * qk[t]) / den;
            }
            ru[t][k * P] = rk[t];
            qu[t][k * P] = qk[t];
            aoa[t] = aob; ana[t] = anb;
            vk[t] = vn[t]; vn[t] = vnn[t];
            e2c[t] = e2n[t]; e4c[t] = e4n[t];
        }
        hoF = hoFn; hnF = hnFn;
        dh = one_h ? 0.f : getm_d2f_approx(ho_n - hn_n);
        ho_n = ho_nn; hn_n = hn_nn;
        nuh_c = nuh_n;
    }
    // bottom layer (:260-267, :291-292), back substitution (:304-307);
    // the old values of level k+1 are read before level k is written
    float vprev[NT], rn[NT], qn[NT];
    S xn[NT];
#pragma unroll
    for (int t = 0; t < NT; t++) {
        const float a3 = -ana[t];
        const float xk = inc_f<S>(vk[t]);
        float a2 = hnF + ana[t];
        float a4 = xk * dh + (-dprev[t]) * (aoa[t] + ana[t]);
        if (SRC && e2[t]) a4 = a4 + e2c[t] * xk;
        if (SRC && e2[t]) a2 = a2 - e2c[t];
        if (SRC && e4[t]) a4 = a4 + e4c[t];
        vprev[t] = (a4 - a3 * qk[t]) / (a2 - a3 * rk[t]);
        xn[t] = v[t][P];
        rn[t] = ru[t][P];
        qn[t] = qu[t][P];
        v[t][0] = inc_add<S>(vk[t], vprev[t]);
    }
    for (k = 1; k < nz; k++) {
#pragma unroll
        for (int t = 0; t < NT; t++) {
            const S x_old = xn[t];
            const float r = rn[t], q = qn[t];
            if (k + 1 < nz) {
                xn[t] = v[t][(k + 1) * P];
                rn[t] = ru[t][(k + 1) * P];
                qn[t] = qu[t][(k + 1) * P];
            }
            vprev[t] = q - r * vprev[t];
            v[t][k * P] = inc_add<S>(x_old, vprev[t]);
        }
    }
}

// PAIRS: fields in pairs (then an odd last one alone), else one at a time.
// Blocks of 32 columns by GETM_TUNE_COLUMN_ROWS rows.  S: storage type of
// the fields (float, or double for FP64 tracer storage).
template <bool SRC, bool PAIRS, typename S = float>
__global__ void __launch_bounds__(128, 7) vd_inc_kernel(VDArgs<float, S> a)
{
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= a.nx_ || j >= a.ny_) return;
    const long long c = (long long)j * a.nx_ + i;
    if (a.nz == 1) {  // diffusion.F90:224-231: every point, mask not consulted
        for (int t = 0; t < a.ntracer; t++) {
            const S x = a.var[t][c];
            const float xf = inc_f<S>(x);
            float a2 = vd_h<float>(a.hn[c]);
            float r = xf * vd_dh(a.ho, a.hn, c);
            if (a.ea2[t]) { a2 = a2 - a.ea2[t][c]; r = r + a.ea2[t][c] * xf; }
            if (a.ea4[t]) r = r + a.ea4[t][c];
            a.var[t][c] = inc_add<S>(x, r / a2);
        }
        return;
    }
    if (a.mask[c] != 1) return;
    int t0 = 0;
    if constexpr (PAIRS)
        for (; t0 + 2 <= a.ntracer; t0 += 2) vd_inc_sweep<2, SRC, S>(a, c, t0);
    for (; t0 < a.ntracer; t0++) vd_inc_sweep<1, SRC, S>(a, c, t0);
}

// ---------------------------------------------------------------------------
// Segmented column solve (mixed form): VD_NSEG warps share 32 columns
// ---------------------------------------------------------------------------
// The partition method for tridiagonal systems (H. H. Wang, ACM Trans. Math.
// Softw. 7 (1981) 170-183), in the thread-per-segment form of the hybrid
// Thomas/PCR solvers (A. Laszlo, M. Giles, J. Appleyard, ACM Trans. Math.
// Softw. 42 (2016) 31).  Warp s of a block owns levels klo..khi (about
// nz / VD_NSEG of them) of the block's 32 columns; lane i is column i, so
// every load and store is still a coalesced 128- or 256-byte row of a level.
// Each thread
//   1. forms the rows of its levels with the arithmetic of vd_inc_sweep
//      (the increment form: A dx = a4 - A x) and, sweeping up, eliminates
//      each row's coupling to the level below in favour of the segment's
//      first unknown, then, sweeping down through shared memory, the
//      coupling to the level above in favour of its last unknown, so that
//      dx_i = d_i - a_i dx_first - g_i dx_last inside the segment;
//   2. adds the rows of its first and last unknown to a reduced tridiagonal
//      system of 2 VD_NSEG unknowns per column, which warp 0 solves by
//      Thomas elimination in shared memory;
//   3. substitutes the two back into its levels and adds the increments to
//      the stored values.
// A column's chain of dependent steps is VD_NSEG times shorter than the
// serial sweep's, and the elimination coefficients stay in shared memory
// (no global workspace).  It costs one reciprocal and about twice the
// multiply-adds per row and level; the rounding differs from the serial
// sweep's by float rounding of the increments.  Used for 2 VD_NSEG <= nz <=
// VD_NSEG * VD_SEG_MAXM when the GETM_TUNE_COLUMN_SOLVE knob asks for it.
constexpr int VD_NSEG = 4;
constexpr int VD_SEG_MAXM = 16;
constexpr int VD_SEG_THREADS = 32 * VD_NSEG;

// Shared memory of one launch: 3 NT (maxm - 2) per-level coefficients per
// thread (levels strictly inside a segment), and the reduced systems of the
// block's 32 columns (lower, diagonal, upper, right-hand side; the solution
// overwrites the right-hand side).
static size_t vd_seg_smem(int nz, int nt)
{
    const int maxm = (nz + VD_NSEG - 1) / VD_NSEG;
    return sizeof(float) * ((size_t)3 * nt * (maxm > 2 ? maxm - 2 : 0) * VD_SEG_THREADS +
                            (size_t)4 * nt * 2 * VD_NSEG * 32);
}

template <int NT, bool SRC, typename S>
__device__ __forceinline__ void vd_seg_group(const VDArgs<float, S>& a, long long c, bool act, int t0, int s,
                                             int klo, int m, int slots, float* __restrict__ rows,
                                             float* __restrict__ red, int tid, int tx)
{
    constexpr int R = 2 * VD_NSEG;
    const long long P = a.plane;
    const int nz = a.nz;
    // coefficient q (0: a, 1: g, 2: d) of field t at inner level ii (1..m-2)
#define VD_ROW(t, q, ii) rows[(((t) * 3 + (q)) * slots + (ii) - 1) * VD_SEG_THREADS + tid]
    // reduced system of this column: q 0 lower, 1 diagonal, 2 upper, 3 rhs
#define VD_RED(t, q, r) red[(((t) * 4 + (q)) * R + (r)) * 32 + tx]
    if (act) {
        const double* __restrict__ ho = a.ho + c;
        const double* __restrict__ hn = a.hn + c;
        const float* __restrict__ nuh = a.nuh + c;
        const bool one_h = a.ho == a.hn;
        const float co = (float)(1.0 - a.cnpar), cn = (float)a.cnpar, dt2 = (float)(2.0 * a.dt);
        S* v[NT];
        const float* e2[NT];
        const float* e4[NT];
        float mol[NT];
#pragma unroll
        for (int t = 0; t < NT; t++) {
            v[t] = a.var[t0 + t] + c;
            e2[t] = SRC && a.ea2[t0 + t] ? a.ea2[t0 + t] + c : nullptr;
            e4[t] = SRC && a.ea4[t0 + t] ? a.ea4[t0 + t] + c : nullptr;
            mol[t] = (float)a.molecular[t0 + t];
        }
        // level k = klo; the interface below it (k >= 1)
        int k = klo;
        float hoF = vd_h<float>(ho[k * P]), hnF = vd_h<float>(hn[k * P]);
        float dh = one_h ? 0.f : getm_d2f_approx(ho[k * P] - hn[k * P]);
        S xc[NT];
        float aob[NT], anb[NT], ddn[NT];
#pragma unroll
        for (int t = 0; t < NT; t++) {
            xc[t] = v[t][k * P];
            aob[t] = anb[t] = ddn[t] = 0.f;
        }
        if (k >= 1) {
            const float hoFb = vd_h<float>(ho[(k - 1) * P]), hnFb = vd_h<float>(hn[(k - 1) * P]);
            const float nb = nuh[k * P];
#pragma unroll
            for (int t = 0; t < NT; t++) {
                const float x = dt2 * (nb + mol[t]);
                aob[t] = co * x / (hoF + hoFb);
                anb[t] = cn * x / (hnF + hnFb);
                ddn[t] = inc_f<S>(v[t][(k - 1) * P] - xc[t]);
            }
        }
        // operands of the level above (k + 1), one level ahead of the arithmetic
        double ho_a = 0.0, hn_a = 0.0;
        float nuh_a = 0.f, e2c[NT], e4c[NT];
        S xa[NT];
        if (k + 1 < nz) {
            ho_a = ho[(k + 1) * P];
            hn_a = hn[(k + 1) * P];
            nuh_a = nuh[(k + 1) * P];
        }
#pragma unroll
        for (int t = 0; t < NT; t++) {
            xa[t] = k + 1 < nz ? v[t][(k + 1) * P] : S(0);
            e2c[t] = SRC && e2[t] ? e2[t][k * P] : 0.f;
            e4c[t] = SRC && e4[t] ? e4[t][k * P] : 0.f;
        }
        float L0[NT], D0[NT], U0[NT], R0[NT], al[NT], ga[NT], de[NT];
        for (int ii = 0; ii < m; ii++, k++) {
            const bool top = k == nz - 1, bot = k == 0;
            // raw operands of level k + 2 and the sources of level k + 1
            double ho_n = 0.0, hn_n = 0.0;
            float nuh_n = 0.f, e2n[NT], e4n[NT];
            S xn[NT];
            if (k + 2 < nz) {
                ho_n = ho[(k + 2) * P];
                hn_n = hn[(k + 2) * P];
                nuh_n = nuh[(k + 2) * P];
            }
#pragma unroll
            for (int t = 0; t < NT; t++) {
                xn[t] = k + 2 < nz ? v[t][(k + 2) * P] : S(0);
                e2n[t] = SRC && e2[t] && k + 1 < nz ? e2[t][(k + 1) * P] : 0.f;
                e4n[t] = SRC && e4[t] && k + 1 < nz ? e4[t][(k + 1) * P] : 0.f;
            }
            const float hoFa = top ? 0.f : vd_h<float>(ho_a), hnFa = top ? 0.f : vd_h<float>(hn_a);
            const float dha = (one_h || top) ? 0.f : getm_d2f_approx(ho_a - hn_a);
#pragma unroll
            for (int t = 0; t < NT; t++) {
                // interface above level k (vd_aux with C level k) and the
                // difference to the level above, as in vd_inc_sweep
                float aoa = 0.f, ana = 0.f, dup = 0.f;
                if (!top) {
                    const float x = dt2 * (nuh_a + mol[t]);
                    aoa = co * x / (hoFa + hoF);
                    ana = cn * x / (hnFa + hnF);
                    dup = inc_f<S>(xa[t] - xc[t]);
                }
                const float xk = inc_f<S>(xc[t]);
                float dg, rh;
                if (top) {
                    dg = hnF + anb[t];
                    rh = xk * dh + ddn[t] * (aob[t] + anb[t]);
                } else if (bot) {
                    dg = hnF + ana;
                    rh = xk * dh + dup * (aoa + ana);
                } else {
                    dg = hnF + ana + anb[t];
                    rh = xk * dh + dup * (aoa + ana) + ddn[t] * (aob[t] + anb[t]);
                }
                if (SRC && e2[t]) rh = rh + e2c[t] * xk;
                if (SRC && e2[t]) dg = dg - e2c[t];
                if (SRC && e4[t]) rh = rh + e4c[t];
                const float lw = bot ? 0.f : -anb[t];
                const float up = top ? 0.f : -ana;
                if (ii == 0) {
                    L0[t] = lw; D0[t] = dg; U0[t] = up; R0[t] = rh;
                } else if (ii == 1) {
                    const float inv = 1.f / dg;
                    al[t] = lw * inv; ga[t] = up * inv; de[t] = rh * inv;
                } else {
                    const float inv = 1.f / (dg - lw * ga[t]);
                    al[t] = -(lw * al[t]) * inv;
                    ga[t] = up * inv;
                    de[t] = (rh - lw * de[t]) * inv;
                }
                if (ii >= 1 && ii < m - 1) {
                    VD_ROW(t, 0, ii) = al[t];
                    VD_ROW(t, 1, ii) = ga[t];
                    VD_ROW(t, 2, ii) = de[t];
                }
                aob[t] = aoa; anb[t] = ana; ddn[t] = -dup;
                xc[t] = xa[t]; xa[t] = xn[t];
                e2c[t] = e2n[t]; e4c[t] = e4n[t];
            }
            hoF = hoFa; hnF = hnFa; dh = dha;
            ho_a = ho_n; hn_a = hn_n; nuh_a = nuh_n;
        }
        // down through the inner levels: dx_ii = d - a dx_first - g dx_last
        float as[NT], gs[NT], ds[NT];
#pragma unroll
        for (int t = 0; t < NT; t++) { as[t] = 0.f; gs[t] = -1.f; ds[t] = 0.f; }
        for (int ii = m - 2; ii >= 1; ii--) {
#pragma unroll
            for (int t = 0; t < NT; t++) {
                const float a_ = VD_ROW(t, 0, ii), g_ = VD_ROW(t, 1, ii), d_ = VD_ROW(t, 2, ii);
                ds[t] = d_ - g_ * ds[t];
                as[t] = a_ - g_ * as[t];
                gs[t] = -(g_ * gs[t]);
                VD_ROW(t, 0, ii) = as[t];
                VD_ROW(t, 1, ii) = gs[t];
                VD_ROW(t, 2, ii) = ds[t];
            }
        }
        // the segment's rows of the reduced system
#pragma unroll
        for (int t = 0; t < NT; t++) {
            VD_RED(t, 0, 2 * s) = L0[t];
            VD_RED(t, 1, 2 * s) = D0[t] - U0[t] * as[t];
            VD_RED(t, 2, 2 * s) = -(U0[t] * gs[t]);
            VD_RED(t, 3, 2 * s) = R0[t] - U0[t] * ds[t];
            VD_RED(t, 0, 2 * s + 1) = al[t];
            VD_RED(t, 1, 2 * s + 1) = 1.f;
            VD_RED(t, 2, 2 * s + 1) = ga[t];
            VD_RED(t, 3, 2 * s + 1) = de[t];
        }
    }
    __syncthreads();
    if (s == 0 && act) {
#pragma unroll
        for (int t = 0; t < NT; t++) {
            float cp[R], dp[R];
            cp[0] = VD_RED(t, 2, 0) / VD_RED(t, 1, 0);
            dp[0] = VD_RED(t, 3, 0) / VD_RED(t, 1, 0);
#pragma unroll
            for (int r = 1; r < R; r++) {
                const float lw = VD_RED(t, 0, r);
                const float inv = 1.f / (VD_RED(t, 1, r) - lw * cp[r - 1]);
                cp[r] = VD_RED(t, 2, r) * inv;
                dp[r] = (VD_RED(t, 3, r) - lw * dp[r - 1]) * inv;
            }
            float x = dp[R - 1];
            VD_RED(t, 3, R - 1) = x;
#pragma unroll
            for (int r = R - 2; r >= 0; r--) {
                x = dp[r] - cp[r] * x;
                VD_RED(t, 3, r) = x;
            }
        }
    }
    __syncthreads();
    if (act) {
#pragma unroll
        for (int t = 0; t < NT; t++) {
            S* __restrict__ vt = a.var[t0 + t] + c;
            const float xF = VD_RED(t, 3, 2 * s), xL = VD_RED(t, 3, 2 * s + 1);
            S xo = vt[klo * P];
            for (int ii = 0; ii < m; ii++) {
                const int k = klo + ii;
                const S xnext = ii + 1 < m ? vt[(k + 1) * P] : S(0);
                const float dx = ii == 0 ? xF
                                 : ii == m - 1 ? xL
                                               : VD_ROW(t, 2, ii) - VD_ROW(t, 0, ii) * xF - VD_ROW(t, 1, ii) * xL;
                vt[k * P] = inc_add<S>(xo, dx);
                xo = xnext;
            }
        }
    }
    __syncthreads();  // shared memory is reused by the next group of fields
#undef VD_ROW
#undef VD_RED
}

// One row j of 32 columns per block (blockIdx.x: 32-column strip, blockIdx.y:
// row); fields in groups of NT (then an odd last one alone).
template <int NT, bool SRC, typename S>
__global__ void __launch_bounds__(VD_SEG_THREADS, 4) vd_seg_kernel(VDArgs<float, S> a)
{
    extern __shared__ __align__(16) unsigned char vd_smem[];
    const int tx = threadIdx.x, s = threadIdx.y, tid = s * 32 + tx;
    const int i = blockIdx.x * 32 + tx, j = blockIdx.y;
    const long long c = (long long)j * a.nx_ + i;
    const bool act = i < a.nx_ && a.mask[c] == 1;
    const int nz = a.nz;
    const int klo = s * nz / VD_NSEG, m = (s + 1) * nz / VD_NSEG - klo;
    const int maxm = (nz + VD_NSEG - 1) / VD_NSEG;
    const int slots = maxm > 2 ? maxm - 2 : 0;
    float* rows = (float*)vd_smem;
    float* red = rows + (size_t)3 * NT * slots * VD_SEG_THREADS;
    int t0 = 0;
    for (; t0 + NT <= a.ntracer; t0 += NT) vd_seg_group<NT, SRC, S>(a, c, act, t0, s, klo, m, slots, rows, red, tid, tx);
    if constexpr (NT > 1)
        for (; t0 < a.ntracer; t0++) vd_seg_group<1, SRC, S>(a, c, act, t0, s, klo, m, slots, rows, red, tid, tx);
}

template <int NT, bool SRC, typename S>
static int vd_seg_launch_one(VDArgs<float, S>& a, cudaStream_t stream)
{
    const size_t smem = vd_seg_smem(a.nz, NT);
    if (smem > 48 * 1024) {
        // nz up to VD_NSEG * VD_SEG_MAXM needs at most ~60 KB
        if (cudaFuncSetAttribute(vd_seg_kernel<NT, SRC, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return GETM_ERR_CUDA;
    }
    const dim3 grid(getm_div_up(a.nx_, 32), a.ny_), block(32, VD_NSEG);
    vd_seg_kernel<NT, SRC, S><<<grid, block, smem, stream>>>(a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// Whether the segmented solve takes this call (knob set, nz in range).
static bool vd_seg_applies(int nz)
{
    return getm_tune(GETM_TUNE_COLUMN_SOLVE) == 1 && nz >= 2 * VD_NSEG && nz <= VD_NSEG * VD_SEG_MAXM;
}

template <typename S>
static int vd_seg_launch(VDArgs<float, S>& a, cudaStream_t stream)
{
    bool src = false;
    for (int t = 0; t < a.ntracer; t++) src = src || a.ea2[t] || a.ea4[t];
    const bool pairs = a.ntracer > 1;
    if (src && pairs) return vd_seg_launch_one<2, true, S>(a, stream);
    if (src) return vd_seg_launch_one<1, true, S>(a, stream);
    if (pairs) return vd_seg_launch_one<2, false, S>(a, stream);
    return vd_seg_launch_one<1, false, S>(a, stream);
}

// The increment-form solve for FP64-stored fields (float solve, nuh and
// sources; work: 2 nz planes of floats per field of a pair).
static int vd_launch_f64s(VDArgs<float, double>& a, cudaStream_t stream)
{
    if (a.nz > 1 && vd_seg_applies(a.nz)) return vd_seg_launch(a, stream);
    if (!a.work) return GETM_ERR_ARG;
    const int rows = getm_tune(GETM_TUNE_COLUMN_ROWS);
    const dim3 grid(getm_div_up(a.nx_, 32), getm_div_up(a.ny_, rows)), block(32, rows);
    bool src = false;
    for (int t = 0; t < a.ntracer; t++) src = src || a.ea2[t] || a.ea4[t];
    const bool pairs = a.ntracer > 1;
    if (src && pairs) vd_inc_kernel<true, true, double><<<grid, block, 0, stream>>>(a);
    else if (src) vd_inc_kernel<true, false, double><<<grid, block, 0, stream>>>(a);
    else if (pairs) vd_inc_kernel<false, true, double><<<grid, block, 0, stream>>>(a);
    else vd_inc_kernel<false, false, double><<<grid, block, 0, stream>>>(a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

// prepare as a separate call (diffusion.F90:163-171): auxo/auxn at every
// point of the halo-inclusive extent, Fortran levels kmin..kmax-1.
__global__ void vd_prepare_kernel(int nx_, int ny_, int nz, long long plane, double molecular,
                                  const double* nuh, double dt, double cnpar, const double* dzo,
                                  const double* dzn, double* auxo, double* auxn)
{
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n = plane * (nz - 1);
    if (p >= n) return;
    int k = (int)(p / plane);
    long long c = p - (long long)k * plane;
    double x = 2.0 * dt * (nuh[c + (k + 1) * plane] + molecular);
    auxo[p] = (1.0 - cnpar) * x / (dzo[c + (k + 1) * plane] + dzo[c + k * plane]);
    auxn[p] = cnpar * x / (dzn[c + (k + 1) * plane] + dzn[c + k * plane]);
}

template <typename T>
static int vd_launch(VDArgs<T>& a, cudaStream_t stream)
{
    if (a.work) {
        dim3 grid(getm_div_up(a.nx_, 128), a.ny_);
        if constexpr (getm_increment_form<T>) {
            if (a.nz > 1 && !a.auxo && vd_seg_applies(a.nz)) return vd_seg_launch(a, stream);
            if (a.nz > 1 && !a.auxo) {
                const int rows = getm_tune(GETM_TUNE_COLUMN_ROWS);
                const dim3 grid(getm_div_up(a.nx_, 32), getm_div_up(a.ny_, rows)), block(32, rows);
                bool src = false;
                for (int t = 0; t < a.ntracer; t++) src = src || a.ea2[t] || a.ea4[t];
                const bool pairs = a.ntracer > 1;
                if (src && pairs) vd_inc_kernel<true, true><<<grid, block, 0, stream>>>(a);
                else if (src) vd_inc_kernel<true, false><<<grid, block, 0, stream>>>(a);
                else if (pairs) vd_inc_kernel<false, true><<<grid, block, 0, stream>>>(a);
                else vd_inc_kernel<false, false><<<grid, block, 0, stream>>>(a);
                GETM_CHECK_LAUNCH();
                return GETM_OK;
            }
        }
        vd_column_kernel<T, true><<<grid, 128, 0, stream>>>(a);
        GETM_CHECK_LAUNCH();
        return GETM_OK;
    }
    int threads = 128;
    const size_t per = (size_t)vd_smem_arrays<T> * a.nz * sizeof(T);
    while (threads > 32 && per * threads > 160 * 1024) threads /= 2;
    size_t smem = per * threads;
    if (smem > 200 * 1024) return GETM_ERR_NZ;
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(vd_column_kernel<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set = true;
    }
    dim3 grid(getm_div_up(a.nx_, threads), a.ny_);
    vd_column_kernel<T, false><<<grid, threads, smem, stream>>>(a);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_vertical_diffusion_create(getm_grid* tgrid, getm_vertical_diffusion** out)
{
    if (!out) return GETM_ERR_ARG;
    getm_vertical_diffusion* d = (getm_vertical_diffusion*)calloc(1, sizeof(*d));
    if (!d) return GETM_ERR_ALLOC;
    d->tgrid = tgrid;
    *out = d;
    return GETM_OK;
}

extern "C" int getm_vertical_diffusion_finalize(getm_vertical_diffusion* d)
{
    if (!d) return GETM_OK;
    cudaFree(d->auxo);
    cudaFree(d->auxn);
    free(d);
    return GETM_OK;
}

extern "C" int getm_vertical_diffusion_prepare(getm_vertical_diffusion* d, int nx, int ny, int nz,
                                               double molecular, const double* nuh,
                                               double timestep, double cnpar, const int* mask,
                                               const double* ho, const double* hn,
                                               cudaStream_t stream)
{
    (void)mask;
    if (!d || nx < 1 || ny < 1 || nz < 1 || !nuh || !ho || !hn) return GETM_ERR_ARG;
    if (nz > GETM_MAX_NZ) return GETM_ERR_NZ;
    if (nz == 1) return GETM_OK;  // diffusion.F90:155
    const long long plane = (long long)nx * ny;
    const size_t n3 = (size_t)plane * nz;
    if (n3 > d->n3) {
        if (d->auxo) cudaFree(d->auxo);  // (cudaFree waits for the whole device)
        if (d->auxn) cudaFree(d->auxn);
        d->auxo = d->auxn = NULL;
        if (cudaMalloc(&d->auxo, n3 * sizeof(double)) != cudaSuccess) return GETM_ERR_ALLOC;
        if (cudaMalloc(&d->auxn, n3 * sizeof(double)) != cudaSuccess) return GETM_ERR_ALLOC;
        d->n3 = n3;
    }
    long long n = plane * (nz - 1);
    vd_prepare_kernel<<<getm_div_up(n, 256), 256, 0, stream>>>(nx, ny, nz, plane, molecular, nuh, timestep, cnpar, ho, hn, d->auxo, d->auxn);
    GETM_CHECK_LAUNCH();
    return GETM_OK;
}

extern "C" int getm_vertical_diffusion_apply(getm_vertical_diffusion* d, int nx, int ny, int nz,
                                             const int* mask, const double* ho, const double* hn,
                                             double* var, const double* ea2, const double* ea4,
                                             cudaStream_t stream)
{
    if (!d || nx < 1 || ny < 1 || nz < 1 || !mask || !ho || !hn || !var) return GETM_ERR_ARG;
    if (nz > GETM_MAX_NZ) return GETM_ERR_NZ;
    if (nz > 1 && (!d->auxo || d->n3 < (size_t)nx * ny * nz)) return GETM_ERR_ARG;  // not prepared
    VDArgs<double> a;
    memset(&a, 0, sizeof(a));
    a.nx_ = nx; a.ny_ = ny; a.nz = nz; a.plane = (long long)nx * ny;
    a.mask = mask; a.ho = ho; a.hn = hn; a.auxo = d->auxo; a.auxn = d->auxn;
    a.ntracer = 1; a.var[0] = var; a.ea2[0] = ea2; a.ea4[0] = ea4;
    return vd_launch(a, stream);
}

template <typename T, typename S = T>
static int vd_batch_impl(int nx, int ny, int nz, const int* mask, const T* nuh, double timestep, double cnpar,
                         const double* ho, const double* hn, int ntracer, const double* molecular,
                         S* const* vars, const T* const* ea2, const T* const* ea4, T* work, cudaStream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || !mask || !nuh || !ho || !hn || ntracer < 1 || !vars || !molecular)
        return GETM_ERR_ARG;
    if (nz > GETM_MAX_NZ) return GETM_ERR_NZ;
    VDArgs<T, S> a;
    memset(&a, 0, sizeof(a));
    a.nx_ = nx; a.ny_ = ny; a.nz = nz; a.plane = (long long)nx * ny;
    a.mask = mask; a.nuh = nuh; a.ho = ho; a.hn = hn; a.dt = timestep; a.cnpar = cnpar;
    a.work = work;
    int done = 0;
    do {
        int n = ntracer - done;
        if (n > VD_MAX_BATCH) n = VD_MAX_BATCH;
        a.ntracer = n;
        for (int t = 0; t < n; t++) {
            a.molecular[t] = molecular[done + t];
            a.var[t] = vars[done + t];
            a.ea2[t] = ea2 ? ea2[done + t] : NULL;
            a.ea4[t] = ea4 ? ea4[done + t] : NULL;
        }
        int rc;
        if constexpr (std::is_same<T, S>::value) rc = vd_launch<T>(a, stream);
        else rc = vd_launch_f64s(a, stream);
        if (rc) return rc;
        done += n;
    } while (done < ntracer);
    return GETM_OK;
}

extern "C" int getm_vertical_diffusion_batch(int nx, int ny, int nz, const int* mask,
                                             const double* nuh, double timestep, double cnpar,
                                             const double* ho, const double* hn, int ntracer,
                                             const double* molecular, double* const* vars,
                                             const double* const* ea2, const double* const* ea4,
                                             double* work, cudaStream_t stream)
{
    return vd_batch_impl<double>(nx, ny, nz, mask, nuh, timestep, cnpar, ho, hn, ntracer, molecular, vars, ea2, ea4,
                                 work, stream);
}

extern "C" int getm_vertical_diffusion_batch_f32(int nx, int ny, int nz, const int* mask, const float* nuh,
                                                 double timestep, double cnpar, const double* ho,
                                                 const double* hn, int ntracer, const double* molecular,
                                                 float* const* vars, const float* const* ea2,
                                                 const float* const* ea4, float* work, cudaStream_t stream)
{
    return vd_batch_impl<float>(nx, ny, nz, mask, nuh, timestep, cnpar, ho, hn, ntracer, molecular, vars, ea2, ea4,
                                work, stream);
}

extern "C" int getm_vertical_diffusion_batch_f64s(int nx, int ny, int nz, const int* mask, const float* nuh,
                                                  double timestep, double cnpar, const double* ho,
                                                  const double* hn, int ntracer, const double* molecular,
                                                  double* const* vars, const float* const* ea2,
                                                  const float* const* ea4, float* work, cudaStream_t stream)
{
    return vd_batch_impl<float, double>(nx, ny, nz, mask, nuh, timestep, cnpar, ho, hn, ntracer, molecular, vars,
                                        ea2, ea4, work, stream);
}
