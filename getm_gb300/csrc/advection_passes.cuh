// Horizontal advection passes as device functions (shared by the one-pass
// kernels of advection.cu and the fused 2D-substep kernel of split2d.cu).
// Reference: src/operators/advection_schemes/advection.F90.template
// (u2d :23-121, v2d :123-221) and limiters.h.
#pragma once

#include "getm_common.cuh"

#define GETM_MAX_BATCH 32
#define GETM_V_BY 16

// ---------------------------------------------------------------------------
// horizontal pass kernels
// ---------------------------------------------------------------------------
// T is the type of the advected fields, V that of the velocities (T unless
// given): double for the FP64 form, float for the mixed form; the mixed form
// with FP64 tracer storage has T = double, V = float (its increments are
// still formed in float).  Layer thicknesses, the transports QU that update
// them and all grid metrics are double in every form.  For T = V = double
// without increment form every expression below is the FP64 reference
// arithmetic.
template <typename T, typename V = T>
struct HPassArgs {
    int nx_, ny_, nk;
    long long plane;            // nx_ * ny_
    int ilo, ihi, jlo, jhi;     // C interior bounds (inclusive) of the T grid
    const int* umask;           // mask of the velocity grid of this direction
    const double* idx;          // x: idx of U grid; y: idy of V grid (Courant number)
    const double* dy;           // x: dy of U grid;  y: dx of V grid (face length)
    const int* tmask;
    const double* iA;
    const double* Ah;           // 2D horizontal diffusivity on the velocity grid, or NULL
    const V* u;                 // velocity (nk layers)
    const double* hu;           // layer thickness on the velocity grid (nk layers)
    const double* h_in;
    double* h_out;
    double dt;
    int scheme;
    int ntracer;
    // mixed form: float copies of dt and of the metrics above; increment != 0
    // selects the increment-form kernels for double fields (2D momentum)
    int increment;
    float dtf;
    int ych;                    // rows a warp marches in the 3D y pass (launch-shape knob)
    const float* idx_f;
    const float* dy_f;
    const float* iA_f;
    const T* fin[GETM_MAX_BATCH];
    T* fout[GETM_MAX_BATCH];
};

// Epilogue of a pass: called once per updated (or copied) cell with the
// cell's flat index p3, its row j, the new value of the first field and the
// new thickness.  The default does nothing; the one-launch 2D substep uses
// it to form the momentum advection term as each cell is finished.
struct NoEpi {
    __device__ __forceinline__ void operator()(long long, int, double, double) const {}
};

template <typename T>
struct FaceGeom {
    double QU;
    T cfl;
    bool active, up, uu_ok;
};

// Face quantities that do not depend on the advected field
// (template :63-65, :70, :77).
template <typename T>
__device__ __forceinline__ FaceGeom<T> face_geom(const HPassArgs<T>& a, long long p2, long long p3,
                                                 long long s, bool in_range)
{
    FaceGeom<T> g;
    g.QU = 0.0; g.cfl = T(0); g.active = false; g.up = false; g.uu_ok = false;
    if (!in_range) return g;
    int m = a.umask[p2];
    if (!getm_flux_point(m)) return g;
    T uu = a.u[p3];
    g.active = true;
    g.QU = (double)uu * a.hu[p3] * a.dy[p2];
    g.cfl = fabs(uu * (T)a.dt * (T)a.idx[p2]);
    g.up = uu > T(0);
    g.uu_ok = getm_flux_point(g.up ? a.umask[p2 - s] : a.umask[p2 + s]);
    return g;
}

// Tracer flux through one face (template :66-104).
template <typename T>
__device__ __forceinline__ T face_flux(const HPassArgs<T>& a, const FaceGeom<T>& g, const T* __restrict__ f,
                                       long long p2, long long p3, long long s)
{
    if (!g.active) return T(0);
    T fu, fuu, fd;
    if (g.up) {
        fu = f[p3];
        fuu = g.uu_ok ? f[p3 - s] : fu;
        fd = f[p3 + s];
    } else {
        fu = f[p3 + s];
        fuu = g.uu_ok ? f[p3 + 2 * s] : fu;
        fd = f[p3];
    }
    fu = getm_tvd_face<T>(a.scheme, fuu, fu, fd, g.cfl);
    T flux = (T)g.QU * fu;
    if (a.Ah) flux = flux - (T)a.Ah[p2] * (T)a.hu[p3] * (f[p3 + s] - f[p3]) * (T)a.idx[p2] * (T)a.dy[p2];
    return flux;
}

// x-direction pass.  blockDim = (32, BYX); grid = (ceil(nx_/32), ceil(ny_*nk/BYX)).
template <typename T, typename Epi = NoEpi>
__device__ __forceinline__ void hpass_x_body(const HPassArgs<T>& a, int bx, long long row, int lane,
                                             const Epi& epi = Epi())
{
    const int i = bx * 32 + lane;
    if (row >= (long long)a.ny_ * a.nk) return;  // whole warp shares one row
    const int k = (int)(row / a.ny_);
    const int j = (int)(row - (long long)k * a.ny_);
    const bool inx = i < a.nx_;
    const long long p2 = (long long)j * a.nx_ + i;
    const long long p3 = (long long)k * a.plane + p2;
    const bool jrow = j >= a.jlo && j <= a.jhi;

    FaceGeom<T> gr = face_geom(a, p2, p3, 1, inx && jrow && i >= a.ilo - 1 && i <= a.ihi);
    FaceGeom<T> gl = face_geom(a, p2 - 1, p3 - 1, 1, lane == 0 && jrow && i - 1 >= a.ilo - 1 && i - 1 <= a.ihi);
    double QUl = __shfl_up_sync(0xffffffffu, gr.QU, 1);
    if (lane == 0) QUl = gl.QU;
    const bool upd = inx && jrow && i >= a.ilo && i <= a.ihi && a.tmask[p2] == 1;

    double hold = 0.0, hnew = 0.0, iA = 0.0;
    if (inx) {
        hold = a.h_in[p3];
        hnew = hold;
        if (upd) {
            iA = a.iA[p2];
            hnew = hold - a.dt * (gr.QU - QUl) * iA;
        }
        a.h_out[p3] = hnew;
    }
    for (int t = 0; t < a.ntracer; t++) {
        const T* __restrict__ f = a.fin[t];
        T fr = inx ? face_flux(a, gr, f, p2, p3, 1) : T(0);
        T fl = __shfl_up_sync(0xffffffffu, fr, 1);
        if (lane == 0) fl = face_flux(a, gl, f, p2 - 1, p3 - 1, 1);
        if (inx) {
            T fo = f[p3];
            T fn = fo;
            if (upd) {
                T hfo = (T)hold * fo;
                T advn = (fr - fl) * (T)iA;
                fn = (hfo - (T)a.dt * advn) / (T)hnew;
            }
            a.fout[t][p3] = fn;
            if (t == 0) epi(p3, j, (double)fn, hnew);
        }
    }
}

// y-direction pass.  blockDim = (32, GETM_V_BY); grid = (ceil(nx_/32), ceil(ny_/BY), nk).
template <typename T, typename Epi = NoEpi>
__device__ __forceinline__ void hpass_y_body(const HPassArgs<T>& a, int bx, int by, int k, int tx, int ty,
                                             double (&sQ)[GETM_V_BY][32], T (&sF)[GETM_V_BY][32],
                                             const Epi& epi = Epi())
{
    const int i = bx * 32 + tx;
    const int j = by * GETM_V_BY + ty;
    const bool in = i < a.nx_ && j < a.ny_;
    const long long s = a.nx_;
    const long long p2 = (long long)j * a.nx_ + i;
    const long long p3 = (long long)k * a.plane + p2;
    const bool icol = i >= a.ilo && i <= a.ihi;

    FaceGeom<T> gt = face_geom(a, p2, p3, s, in && icol && j >= a.jlo - 1 && j <= a.jhi);
    FaceGeom<T> gb = face_geom(a, p2 - s, p3 - s, s, in && ty == 0 && icol && j - 1 >= a.jlo - 1 && j - 1 <= a.jhi);
    sQ[ty][tx] = gt.QU;
    __syncthreads();
    double QUb = ty > 0 ? sQ[ty - 1][tx] : gb.QU;
    const bool upd = in && icol && j >= a.jlo && j <= a.jhi && a.tmask[p2] == 1;

    double hold = 0.0, hnew = 0.0, iA = 0.0;
    if (in) {
        hold = a.h_in[p3];
        hnew = hold;
        if (upd) {
            iA = a.iA[p2];
            hnew = hold - a.dt * (gt.QU - QUb) * iA;
        }
        a.h_out[p3] = hnew;
    }
    for (int t = 0; t < a.ntracer; t++) {
        const T* __restrict__ f = a.fin[t];
        T ft = in ? face_flux(a, gt, f, p2, p3, s) : T(0);
        T fb = (ty == 0 && in) ? face_flux(a, gb, f, p2 - s, p3 - s, s) : T(0);
        __syncthreads();  // previous tracer's reads of sF are done
        sF[ty][tx] = ft;
        __syncthreads();
        if (ty > 0) fb = sF[ty - 1][tx];
        if (in) {
            T fo = f[p3];
            T fn = fo;
            if (upd) {
                T hfo = (T)hold * fo;
                T advn = (ft - fb) * (T)iA;
                fn = (hfo - (T)a.dt * advn) / (T)hnew;
            }
            a.fout[t][p3] = fn;
            if (t == 0) epi(p3, j, (double)fn, hnew);
        }
    }
}

// ---------------------------------------------------------------------------
// Mixed form (float fields): increment form of the same passes.
//
// With hold - hnew = dt iA (QU_e - QU_w), the reference update
// (hold f - dt iA (QU_e f_e - QU_w f_w)) / hnew equals
//     f - dt iA (QU_e (f_e - f) - QU_w (f_w - f)) / hnew
// exactly, where f_e, f_w are the limited face values.  Each face therefore
// provides QU (face - left cell) and QU (face - right cell), formed from
// differences of neighbouring values, so float32 rounding scales with the
// change of the field, a field at rest is reproduced exactly, and the only
// FP64 operations per cell are the thickness update hnew = hold - dh.
// ---------------------------------------------------------------------------
// Storage type S of the advected field and of the velocities: float (the 3D
// fields of the mixed form) or double (the 2D depth-averaged momentum of the
// mixed form, whose state stays FP64 while its increments are evaluated in
// float).  Differences of neighbouring values are formed in S and then
// narrowed, so they keep their accuracy when the values are close.

// Limited face deviation from the upwind cell, given d = f[b] - f[a] across
// the face and the differences on either side, dprev = f[a] - f[a-1] and
// dnext = f[b+1] - f[b]; tf: the face's limiter constants.
__device__ __forceinline__ float hx_dev(const TvdFaceF& tf, bool up, bool uu_ok, float dprev, float d, float dnext)
{
    return up ? getm_tvd_dev_f(tf, d, uu_ok ? dprev : 0.f) : getm_tvd_dev_f(tf, -d, uu_ok ? -dnext : 0.f);
}

// x-direction pass in increment form.  A warp owns one row segment: lane L
// computes the face at U point a = i0 - 1 + L (between cells a and a+1) and,
// for L < 31, updates cell a + 1, whose east face comes from lane L + 1 by a
// shuffle; segments therefore advance by 31 cells.  Every lane runs the same
// instructions (no per-lane special paths): each field is read with one
// coalesced load per warp plus one load of the three values just outside
// the segment (lanes 0-2), and all loads of a lane are independent.
constexpr int HX_STRIDE = 31;

// KB layers k0 .. k0+KB-1 (those below nk) of row j: the 2D fields (masks,
// metrics) are loaded once for all of them, and every load of the KB layers
// is issued before any value is used.
template <typename S, int KB, typename Epi = NoEpi, typename V = S>
__device__ __forceinline__ void hpass_x_inc_rows(const HPassArgs<S, V>& a, int bx, int j, int k0, int lane,
                                                 const Epi& epi = Epi())
{
    constexpr unsigned FULL = 0xffffffffu;
    const int i0 = bx * HX_STRIDE;
    const int ia = i0 - 1 + lane;  // this lane's face (U point) and its west cell
    const int ib = ia + 1;         // the cell this lane updates (lanes 0-30)
    const long long r2 = (long long)j * a.nx_;
    const bool jrow = j >= a.jlo && j <= a.jhi;
    const bool ain = ia >= 0 && ia < a.nx_;
    // lanes 0-2 address the points i0-2, i0+31, i0+32 just outside the lanes' range
    const int ix = lane == 0 ? i0 - 2 : i0 + 30 + lane;
    const bool xin = lane < 3 && ix >= 0 && ix < a.nx_;
    const bool bin = lane < HX_STRIDE && ib < a.nx_;
    // in-bounds copies of the indices for the loads
    const int iac = min(max(ia, 0), a.nx_ - 1), ixc = min(max(ix, 0), a.nx_ - 1), ibc = min(ib, a.nx_ - 1);
    const int um_raw = a.umask[r2 + iac];
    const int umx_raw = a.umask[r2 + ixc];
    const float dyf = a.dy_f[r2 + iac], idxf = a.idx_f[r2 + iac];
    const float ahraw = a.Ah ? getm_d2f_approx(a.Ah[r2 + iac]) : 0.f;
    const int tm = a.tmask[r2 + ibc];
    const float iaf = a.iA_f[r2 + ibc];
    V uraw[KB];
    double huraw[KB], hold[KB];
#pragma unroll
    for (int kk = 0; kk < KB; kk++) {
        const long long r3 = (long long)min(k0 + kk, a.nk - 1) * a.plane + r2;
        uraw[kk] = a.u[r3 + iac];
        huraw[kk] = a.hu[r3 + iac];
        hold[kk] = a.h_in[r3 + ibc];
    }
    const int ntg = a.ntracer < 2 ? a.ntracer : 2;  // tracers of the first group
    S fa_[KB][2], fx_[KB][2];
#pragma unroll
    for (int kk = 0; kk < KB; kk++) {
        const long long r3 = (long long)min(k0 + kk, a.nk - 1) * a.plane + r2;
#pragma unroll
        for (int q = 0; q < 2; q++) {
            if (q < ntg) {
                const S* __restrict__ f = a.fin[q] + r3;
                fa_[kk][q] = f[iac];
                fx_[kk][q] = f[ixc];
            } else {
                fa_[kk][q] = S(0);
                fx_[kk][q] = S(0);
            }
        }
    }

    // face masks (the same for every layer)
    const bool f_in = ain && jrow && ia >= a.ilo - 1 && ia <= a.ihi;
    const int um = ain ? um_raw : 0;
    const int umx = xin ? umx_raw : 0;
    int um_w = __shfl_up_sync(FULL, um, 1), um_e = __shfl_down_sync(FULL, um, 1);
    const int umx0 = __shfl_sync(FULL, umx, 0), umx1 = __shfl_sync(FULL, umx, 1);
    if (lane == 0) um_w = umx0;
    if (lane == 31) um_e = umx1;
    const bool act = f_in && getm_flux_point(um);
    const bool upd = bin && jrow && ib >= a.ilo && ib <= a.ihi && tm == 1;

#pragma unroll
    for (int kk = 0; kk < KB; kk++) {
        if (k0 + kk >= a.nk) break;
        const long long r3 = (long long)(k0 + kk) * a.plane + r2;
        float QU = 0.f, cfl = 0.f, ahd = 0.f;
        bool up = false, uu_ok = false;
        if (act) {
            const float uu = inc_f<V>(uraw[kk]);
            const float huf = getm_d2f_approx(huraw[kk]);
            QU = uu * huf * dyf;
            cfl = fabsf(uu * a.dtf * idxf);
            up = uu > 0.f;
            uu_ok = getm_flux_point(up ? um_w : um_e);
            if (a.Ah) ahd = -ahraw * huf * idxf * dyf;
        }
        const float QUe = __shfl_down_sync(FULL, QU, 1);  // east face of cell ib

        // thickness update of cell ib
        float coef = 0.f;  // dt iA / hnew
        double hnew = hold[kk];
        if (bin) {
            if (upd) {
                const float dh = a.dtf * (QUe - QU) * iaf;
                hnew = hold[kk] - getm_f2d(dh);
                coef = a.dtf * iaf / (getm_d2f_approx(hold[kk]) - dh);
            }
            a.h_out[r3 + ib] = hnew;
        }
        const TvdFaceF tf = getm_tvd_face_f(a.scheme, cfl);
        // tracers two at a time (the first two preloaded with the layer)
        for (int t = 0; t < a.ntracer; t += 2) {
            const int nt = a.ntracer - t >= 2 ? 2 : 1;
            S fa2[2], fx2[2];
            if (t == 0) {
                fa2[0] = fa_[kk][0]; fa2[1] = fa_[kk][1];
                fx2[0] = fx_[kk][0]; fx2[1] = fx_[kk][1];
            } else {
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const S* __restrict__ f = a.fin[t + (q < nt ? q : 0)] + r3;
                    fa2[q] = f[iac];
                    fx2[q] = f[ixc];
                }
            }
#pragma unroll
            for (int q = 0; q < 2; q++) {
                if (q >= nt) break;
                const S fa = ain ? fa2[q] : S(0);
                const S fx = xin ? fx2[q] : S(0);
                S fb = __shfl_down_sync(FULL, fa, 1);  // f[ia+1]
                const S x0 = __shfl_sync(FULL, fx, 0), x1 = __shfl_sync(FULL, fx, 1), x2 = __shfl_sync(FULL, fx, 2);
                if (lane == 31) fb = x1;
                const float d = inc_f<S>(fb - fa);
                float dprev = __shfl_up_sync(FULL, d, 1), dnext = __shfl_down_sync(FULL, d, 1);
                // the two differences the shuffles cannot supply, in one operation
                const float e = inc_f<S>(lane == 0 ? fa - x0 : x2 - x1);
                if (lane == 0) dprev = e;
                if (lane == 31) dnext = e;
                // el = QU (face - f[ia]) (east side of cell ia), er = QU (face - f[ib])
                float el = 0.f, er = 0.f;
                if (act) {
                    const float dev = hx_dev(tf, up, uu_ok, dprev, d, dnext);
                    const float fd = ahd * d;
                    el = QU * (up ? dev : d + dev) + fd;
                    er = QU * (up ? dev - d : dev) + fd;
                }
                const float el_e = __shfl_down_sync(FULL, el, 1);  // east face of cell ib, seen from ib
                if (bin) {
                    const S fn = upd ? inc_add<S>(fb, -coef * (el_e - er)) : fb;
                    a.fout[t + q][r3 + ib] = fn;
                    if (t + q == 0) epi(r3 + ib, j, (double)fn, hnew);
                }
            }
        }
    }
}

// x pass in increment form with four cells per lane, for the 3D passes.  A
// warp sweeps one row (layer k, row j) from west to east in chunks of 128
// cells; lane L of a chunk owns cells i0 + 4L .. i0 + 4L + 3 and their east
// faces, so every load and store of the lane is one 16-byte vector (two for
// doubles) at an aligned address (the caller checks nx_ % 4 == 0 and the
// pointers' alignment).  A face needs the values of the lanes beside it
// (shuffles), the chunk to the west hands its last face over in registers,
// and the last lane reads the two cells east of the chunk.  Each difference
// of neighbouring values is formed once (it serves the face and, in the
// limiter, both faces beside it: one FP64 subtraction per cell and field
// instead of two for FP64 storage).  Every face and cell is evaluated with
// the same expressions as hpass_x_inc_rows, so both give the same bits.
// Fields are swept two at a time (the thickness is written by the first
// sweep).
template <typename T>
__device__ __forceinline__ void xv_load4(const T* p, T (&o)[4])
{
    if constexpr (sizeof(T) == 8) {
        const double2 a = *reinterpret_cast<const double2*>(p);
        const double2 b = *reinterpret_cast<const double2*>(p + 2);
        o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
    } else if constexpr (std::is_same<T, int>::value) {
        const int4 a = *reinterpret_cast<const int4*>(p);
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    } else {
        const float4 a = *reinterpret_cast<const float4*>(p);
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    }
}

template <typename T>
__device__ __forceinline__ void xv_store4(T* p, const T (&v)[4])
{
    if constexpr (sizeof(T) == 8) {
        *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
        *reinterpret_cast<double2*>(p + 2) = make_double2(v[2], v[3]);
    } else {
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
}

constexpr int XV_CHUNK = 128;

template <typename S, typename V = S>
__device__ __forceinline__ void hpass_x_vec_row(const HPassArgs<S, V>& a, int j, int k, int lane)
{
    constexpr unsigned FULL = 0xffffffffu;
    const int nx = a.nx_;
    const long long r2 = (long long)j * nx;
    const long long r3 = (long long)k * a.plane + r2;
    const bool jrow = j >= a.jlo && j <= a.jhi;
    const int ngroup = a.ntracer > 0 ? (a.ntracer + 1) / 2 : 1;
    for (int g = 0; g < ngroup; g++) {
        const int t0 = 2 * g;
        const int nt = a.ntracer - t0 >= 2 ? 2 : a.ntracer - t0;  // 0 with no fields
        // the west face of the chunk's first cell: the chunk to the west's
        // last face (nothing west of the row: an inactive face)
        float cQU = 0.f;
        int cum = 0;
        float cd[2] = {0.f, 0.f}, cer[2] = {0.f, 0.f};
        for (int i0 = 0; i0 < nx; i0 += XV_CHUNK) {
            const int ib = i0 + 4 * lane;  // the lane's first cell and its east face
            const bool lin = ib < nx;      // all four cells or none
            const int ie = i0 + XV_CHUNK;  // the first cell east of the chunk
            int um[4] = {0, 0, 0, 0}, tm[4] = {0, 0, 0, 0};
            float dyf[4] = {0.f, 0.f, 0.f, 0.f}, idxf[4] = {0.f, 0.f, 0.f, 0.f}, iaf[4] = {0.f, 0.f, 0.f, 0.f};
            float ahraw[4] = {0.f, 0.f, 0.f, 0.f};
            V uraw[4] = {V(0), V(0), V(0), V(0)};
            double huraw[4] = {0.0, 0.0, 0.0, 0.0}, hold[4] = {0.0, 0.0, 0.0, 0.0};
            if (lin) {
                xv_load4(a.umask + r2 + ib, um);
                xv_load4(a.tmask + r2 + ib, tm);
                xv_load4(a.dy_f + r2 + ib, dyf);
                xv_load4(a.idx_f + r2 + ib, idxf);
                xv_load4(a.iA_f + r2 + ib, iaf);
                xv_load4(a.u + r3 + ib, uraw);
                xv_load4(a.hu + r3 + ib, huraw);
                xv_load4(a.h_in + r3 + ib, hold);
                if (a.Ah) {
                    double ah[4];
                    xv_load4(a.Ah + r2 + ib, ah);
#pragma unroll
                    for (int m = 0; m < 4; m++) ahraw[m] = getm_d2f_approx(ah[m]);
                }
            }
            // masks of the velocity points beside the lane's first and last faces
            int umW = __shfl_up_sync(FULL, um[3], 1), umE = __shfl_down_sync(FULL, um[0], 1);
            if (lane == 0) umW = cum;
            if (lane == 31) umE = ie < nx ? a.umask[r2 + ie] : 0;

            // face geometry (the same expressions as hpass_x_inc_rows)
            float QU[4], cfl[4], ahd[4];
            bool up[4], uu_ok[4], act[4];
#pragma unroll
            for (int m = 0; m < 4; m++) {
                const int ia = ib + m;
                const bool f_in = lin && jrow && ia >= a.ilo - 1 && ia <= a.ihi;
                act[m] = f_in && getm_flux_point(um[m]);
                QU[m] = 0.f; cfl[m] = 0.f; ahd[m] = 0.f;
                up[m] = false; uu_ok[m] = false;
                if (act[m]) {
                    const float uu = inc_f<V>(uraw[m]);
                    const float huf = getm_d2f_approx(huraw[m]);
                    QU[m] = uu * huf * dyf[m];
                    cfl[m] = fabsf(uu * a.dtf * idxf[m]);
                    up[m] = uu > 0.f;
                    const int mw = m > 0 ? um[m - 1] : umW, me = m < 3 ? um[m + 1] : umE;
                    uu_ok[m] = getm_flux_point(up[m] ? mw : me);
                    if (a.Ah) ahd[m] = -ahraw[m] * huf * idxf[m] * dyf[m];
                }
            }
            float QUw0 = __shfl_up_sync(FULL, QU[3], 1);  // west face of the lane's first cell
            if (lane == 0) QUw0 = cQU;

            // thickness update of the lane's cells
            float coef[4];
            bool upd[4];
            double hnew[4];
#pragma unroll
            for (int m = 0; m < 4; m++) {
                const int c = ib + m;
                upd[m] = lin && jrow && c >= a.ilo && c <= a.ihi && tm[m] == 1;
                coef[m] = 0.f;
                hnew[m] = hold[m];
                if (upd[m]) {
                    const float QUw = m > 0 ? QU[m - 1] : QUw0;
                    const float dh = a.dtf * (QU[m] - QUw) * iaf[m];
                    hnew[m] = hold[m] - getm_f2d(dh);
                    coef[m] = a.dtf * iaf[m] / (getm_d2f_approx(hold[m]) - dh);
                }
            }
            if (g == 0 && lin) xv_store4(a.h_out + r3 + ib, hnew);

#pragma unroll
            for (int q = 0; q < 2; q++) {
                if (q >= nt) break;
                const S* __restrict__ f = a.fin[t0 + q] + r3;
                S fv[4] = {S(0), S(0), S(0), S(0)};
                if (lin) xv_load4(f + ib, fv);
                S fE0 = S(0), fE1 = S(0);  // the two cells east of the chunk (last lane)
                if (lane == 31) {
                    if (ie < nx) fE0 = f[ie];
                    if (ie + 1 < nx) fE1 = f[ie + 1];
                }
                S fn0 = __shfl_down_sync(FULL, fv[0], 1);
                if (lane == 31) fn0 = fE0;
                // differences of neighbouring values in the storage type, then
                // narrowed (d[m]: across face m)
                float d[4];
                d[0] = inc_f<S>(fv[1] - fv[0]);
                d[1] = inc_f<S>(fv[2] - fv[1]);
                d[2] = inc_f<S>(fv[3] - fv[2]);
                d[3] = inc_f<S>(fn0 - fv[3]);
                float dW = __shfl_up_sync(FULL, d[3], 1), dE = __shfl_down_sync(FULL, d[0], 1);
                if (lane == 0) dW = cd[q];
                if (lane == 31) dE = inc_f<S>(fE1 - fE0);
                float el[4], er[4];
#pragma unroll
                for (int m = 0; m < 4; m++) {
                    el[m] = 0.f; er[m] = 0.f;
                    if (act[m]) {
                        const TvdFaceF tf = getm_tvd_face_f(a.scheme, cfl[m]);
                        const float dprev = m > 0 ? d[m - 1] : dW, dnext = m < 3 ? d[m + 1] : dE;
                        const float dev = hx_dev(tf, up[m], uu_ok[m], dprev, d[m], dnext);
                        const float fd = ahd[m] * d[m];
                        el[m] = QU[m] * (up[m] ? dev : d[m] + dev) + fd;
                        er[m] = QU[m] * (up[m] ? dev - d[m] : dev) + fd;
                    }
                }
                float erW = __shfl_up_sync(FULL, er[3], 1);  // west face of the lane's first cell
                if (lane == 0) erW = cer[q];
                S out[4];
#pragma unroll
                for (int m = 0; m < 4; m++) {
                    const float ew = m > 0 ? er[m - 1] : erW;
                    out[m] = upd[m] ? inc_add<S>(fv[m], -coef[m] * (el[m] - ew)) : fv[m];
                }
                if (lin) xv_store4(a.fout[t0 + q] + r3 + ib, out);
                cd[q] = __shfl_sync(FULL, d[3], 31);
                cer[q] = __shfl_sync(FULL, er[3], 31);
            }
            cQU = __shfl_sync(FULL, QU[3], 31);
            cum = __shfl_sync(FULL, um[3], 31);
        }
    }
}

// One row (layer k, row j) of the x pass: row = k ny_ + j.
template <typename S, typename Epi = NoEpi, typename V = S>
__device__ __forceinline__ void hpass_x_inc_body(const HPassArgs<S, V>& a, int bx, long long row, int lane,
                                                 const Epi& epi = Epi())
{
    if (row >= (long long)a.ny_ * a.nk) return;  // whole warp shares one row
    const int k = (int)(row / a.ny_);
    const int j = (int)(row - (long long)k * a.ny_);
    hpass_x_inc_rows<S, 1, Epi, V>(a, bx, j, k, lane, epi);
}

// y-direction pass in increment form: the transpose of hpass_x_inc_kernel.
// A block of 32 x HY_BY threads covers 32 columns; thread row ty computes the
// face at V point ja = j0 - 1 + ty and, for ty < HY_BY - 1, updates cell
// ja + 1, whose north face comes from thread row ty + 1 through shared
// memory; blocks therefore advance by HY_BY - 1 rows.  The rows of each
// tracer a block needs are staged in shared memory once (one coalesced load
// per row), so every value is read from global memory once per block.
constexpr int HY_BY = 16;
constexpr int HY_STRIDE = HY_BY - 1;

template <typename S>
struct YIncSmem {
    S sf[HY_BY + 3][32];       // rows j0-2 .. j0+HY_BY
    float sd[HY_BY + 2][32];   // differences f[j+1] - f[j], rows j0-2 .. j0+HY_BY-1
    float sx[HY_BY][32];       // per-face exchange (QU, then el)
};

template <typename S, typename Epi = NoEpi, typename V = S>
__device__ __forceinline__ void hpass_y_inc_body(const HPassArgs<S, V>& a, int bx, int by, int k, int tx, int ty,
                                                 YIncSmem<S>& sm, const Epi& epi = Epi())
{
    auto& sf = sm.sf;
    auto& sd = sm.sd;
    auto& sx = sm.sx;
    const int i = bx * 32 + tx;
    const int j0 = by * HY_STRIDE;
    const int ja = j0 - 1 + ty;  // this thread's face (V point) and its south cell
    const int jb = ja + 1;       // the cell this thread updates (ty < HY_STRIDE)
    const long long s = a.nx_;
    const long long base = (long long)k * a.plane + i;  // + j * s
    const bool icol = i < a.nx_;
    const bool ain = icol && ja >= 0 && ja < a.ny_;
    const bool iint = i >= a.ilo && i <= a.ihi;

    // face geometry
    const bool f_in = ain && iint && ja >= a.jlo - 1 && ja <= a.jhi;
    float QU = 0.f, cfl = 0.f, ahd = 0.f;
    bool up = false, uu_ok = false, act = false;
    if (f_in) {
        const long long q2 = (long long)ja * s + i;
        act = getm_flux_point(a.umask[q2]);
        if (act) {
            const int m_s = ja > 0 ? a.umask[q2 - s] : 0;
            const int m_n = ja + 1 < a.ny_ ? a.umask[q2 + s] : 0;
            const float vv = inc_f<V>(a.u[base + ja * s]);
            const float hvf = getm_d2f_approx(a.hu[base + ja * s]);
            const float dxf = a.dy_f[q2], idyf = a.idx_f[q2];
            QU = vv * hvf * dxf;
            cfl = fabsf(vv * a.dtf * idyf);
            up = vv > 0.f;
            uu_ok = getm_flux_point(up ? m_s : m_n);
            if (a.Ah) ahd = -getm_d2f_approx(a.Ah[q2]) * hvf * idyf * dxf;
        }
    }
    sx[ty][tx] = QU;
    __syncthreads();
    const float QUn = ty + 1 < HY_BY ? sx[ty + 1][tx] : 0.f;  // north face of cell jb

    const bool bin = ty < HY_STRIDE && icol && jb < a.ny_;
    const bool upd = bin && iint && jb >= a.jlo && jb <= a.jhi && a.tmask[(long long)jb * s + i] == 1;
    float coef = 0.f;
    double hnew = 0.0;
    if (bin) {
        const double hold = a.h_in[base + jb * s];
        hnew = hold;
        if (upd) {
            const float iaf = a.iA_f[(long long)jb * s + i];
            const float dh = a.dtf * (QUn - QU) * iaf;
            hnew = hold - getm_f2d(dh);
            coef = a.dtf * iaf / (getm_d2f_approx(hold) - dh);
        }
        a.h_out[base + jb * s] = hnew;
    }
    // staging rows: thread row ty loads row ja (smem row ty + 1); rows 0-2
    // also load rows j0-2, j0+HY_BY-1 and j0+HY_BY (smem rows 0, HY_BY+1, HY_BY+2)
    const int jx = ty == 0 ? j0 - 2 : j0 + HY_BY - 2 + ty;
    const int sxrow = ty == 0 ? 0 : HY_BY + ty;
    const bool xin = ty < 3 && icol && jx >= 0 && jx < a.ny_;
    const TvdFaceF tf = getm_tvd_face_f(a.scheme, cfl);
    for (int t = 0; t < a.ntracer; t++) {
        const S* __restrict__ f = a.fin[t] + base;
        __syncthreads();  // previous tracer's reads of sf, sd and sx are done
        sf[ty + 1][tx] = ain ? f[ja * s] : S(0);
        if (ty < 3) sf[sxrow][tx] = xin ? f[jx * s] : S(0);
        __syncthreads();
        // difference across this thread's face (smem row ty + 1 of sd); rows
        // 0 and 1 also form the differences below and above the block's faces
        sd[ty + 1][tx] = inc_f<S>(sf[ty + 2][tx] - sf[ty + 1][tx]);
        if (ty == 0) sd[0][tx] = inc_f<S>(sf[1][tx] - sf[0][tx]);
        if (ty == 1) sd[HY_BY + 1][tx] = inc_f<S>(sf[HY_BY + 2][tx] - sf[HY_BY + 1][tx]);
        __syncthreads();
        const float dprev = sd[ty][tx], d = sd[ty + 1][tx], dnext = sd[ty + 2][tx];
        const S fb = sf[ty + 2][tx];
        float el = 0.f, er = 0.f;
        if (act) {
            const float dev = hx_dev(tf, up, uu_ok, dprev, d, dnext);
            const float fd = ahd * d;
            el = QU * (up ? dev : d + dev) + fd;
            er = QU * (up ? dev - d : dev) + fd;
        }
        sx[ty][tx] = el;
        __syncthreads();
        const float el_n = ty + 1 < HY_BY ? sx[ty + 1][tx] : 0.f;
        if (bin) {
            const S fn = upd ? inc_add<S>(fb, -coef * (el_n - er)) : fb;
            a.fout[t][base + jb * s] = fn;
            if (t == 0) epi(base + jb * s, jb, (double)fn, hnew);
        }
    }
}


// y-direction pass in increment form, marching north.  A warp owns 32
// columns of one layer and a chunk of a.ych cells along y.  Walking the
// faces j = j0-1 .. j0+a.ych-1 it keeps the last four rows of every tracer,
// the three differences around the face and the south face's QU and er in
// registers, so each step issues one independent load per field and row
// (no shared memory, no block barriers) and updates cell j from its south
// face (the previous step) and its north face (this step).  The arithmetic
// is that of hpass_y_inc_body, operation for operation; NT tracers are
// marched together, larger batches in groups of NT (the face geometry is
// reloaded per group).

template <typename S, int NT, typename V = S>
__device__ __forceinline__ void hpass_y_march_body(const HPassArgs<S, V>& a, int bx, int chunk, int k, int lane,
                                                   int t0)
{
    const int i = bx * 32 + lane;
    const long long s = a.nx_;
    const bool icol = i < a.nx_;
    const int ic = icol ? i : a.nx_ - 1;  // in-bounds column for the loads of idle lanes
    const long long base = (long long)k * a.plane + ic;
    const bool iint = icol && i >= a.ilo && i <= a.ihi;
    const int jc0 = chunk * a.ych;
    const int jc1 = min(jc0 + a.ych, a.ny_);
    const int nt = min(NT, a.ntracer - t0);
    const bool first_group = t0 == 0;
    // tracers q >= nt of the group (none when ntracer is 0) read as zero
    const S* f[NT];
    S* fo[NT];
#pragma unroll
    for (int q = 0; q < NT; q++) {
        f[q] = q < nt ? a.fin[t0 + q] + base : nullptr;
        fo[q] = q < nt ? a.fout[t0 + q] + base : nullptr;
    }
    auto rowv = [&](const S* p, int j) -> S {
        return (p && j >= 0 && j < a.ny_ && icol) ? p[(long long)j * s] : S(0);
    };
    auto umask_at = [&](int j) -> int { return (j >= 0 && j < a.ny_) ? a.umask[(long long)j * s + ic] : 0; };

    // window at the first face j = jc0 - 1: rows j-1 .. j+1 and d(j-1), d(j)
    S fm1[NT], f0[NT], f1[NT];
    float dm1[NT], d0[NT], er_s[NT];
#pragma unroll
    for (int q = 0; q < NT; q++) {
        fm1[q] = rowv(f[q], jc0 - 2);
        f0[q] = rowv(f[q], jc0 - 1);
        f1[q] = rowv(f[q], jc0);
        dm1[q] = inc_f<S>(f0[q] - fm1[q]);
        d0[q] = inc_f<S>(f1[q] - f0[q]);
        er_s[q] = 0.f;
    }
    int m_m = umask_at(jc0 - 2), m_0 = umask_at(jc0 - 1);
    float QU_s = 0.f;
    // every load of step j
    struct StepLoads {
        int m_1, tm;
        S f2[NT];
        V uraw;
        double huraw, hold;
        float dxf, idyf, ahraw, iaf;
    };
    auto load_step = [&](int j) -> StepLoads {
        StepLoads L;
        L.m_1 = umask_at(j + 1);
#pragma unroll
        for (int q = 0; q < NT; q++) L.f2[q] = rowv(f[q], j + 2);
        const long long jr = (long long)((j >= 0 && j < a.ny_) ? j : 0) * s;
        L.uraw = a.u[base + jr];
        L.huraw = a.hu[base + jr];
        L.dxf = a.dy_f[jr + ic];
        L.idyf = a.idx_f[jr + ic];
        L.ahraw = a.Ah ? getm_d2f_approx(a.Ah[jr + ic]) : 0.f;
        L.hold = a.h_in[base + jr];
        L.tm = a.tmask[jr + ic];
        L.iaf = a.iA_f[jr + ic];
        return L;
    };
    // one tracer: prefetch a step ahead (more loads in flight per warp);
    // two: the registers go to occupancy instead
    constexpr bool PF = NT == 1;
    StepLoads nxt = load_step(jc0 - 1);
    for (int j = jc0 - 1; j < jc1; j++) {
        const StepLoads cur = PF ? nxt : load_step(j);
        if (PF) nxt = load_step(min(j + 1, jc1 - 1));
        const int m_1 = cur.m_1;
        const S* f2 = cur.f2;
        const bool jin = j >= 0 && j < a.ny_;
        const long long jr = (long long)(jin ? j : 0) * s;
        const V uraw = cur.uraw;
        const double huraw = cur.huraw;
        const float dxf = cur.dxf, idyf = cur.idyf, ahraw = cur.ahraw;
        const double hold = cur.hold;
        const int tm = cur.tm;
        const float iaf = cur.iaf;

        // face j (between cells j and j+1)
        const bool f_in = jin && iint && j >= a.jlo - 1 && j <= a.jhi;
        float QU = 0.f, cfl = 0.f, ahd = 0.f;
        bool up = false, uu_ok = false, act = false;
        if (f_in) {
            act = getm_flux_point(m_0);
            if (act) {
                const float vv = inc_f<V>(uraw);
                const float hvf = getm_d2f_approx(huraw);
                QU = vv * hvf * dxf;
                cfl = fabsf(vv * a.dtf * idyf);
                up = vv > 0.f;
                uu_ok = getm_flux_point(up ? m_m : m_1);
                if (a.Ah) ahd = -ahraw * hvf * idyf * dxf;
            }
        }
        // cell j: south face j-1 (previous step), north face j (this step)
        const bool upd_cell = j >= jc0 && iint && j >= a.jlo && j <= a.jhi && tm == 1;
        float coef = 0.f;
        double hnew = hold;
        if (upd_cell) {
            const float dh = a.dtf * (QU - QU_s) * iaf;
            hnew = hold - getm_f2d(dh);
            coef = a.dtf * iaf / (getm_d2f_approx(hold) - dh);
        }
        if (j >= jc0 && icol && first_group) a.h_out[base + jr] = hnew;
        const TvdFaceF tf = getm_tvd_face_f(a.scheme, cfl);
#pragma unroll
        for (int q = 0; q < NT; q++) {
            const float d1 = inc_f<S>(f2[q] - f1[q]);
            float el = 0.f, er = 0.f;
            if (act) {
                const float dev = hx_dev(tf, up, uu_ok, dm1[q], d0[q], d1);
                const float fd = ahd * d0[q];
                el = QU * (up ? dev : d0[q] + dev) + fd;
                er = QU * (up ? dev - d0[q] : dev) + fd;
            }
            if (j >= jc0 && icol && q < nt) fo[q][jr] = upd_cell ? inc_add<S>(f0[q], -coef * (el - er_s[q])) : f0[q];
            er_s[q] = er;
            fm1[q] = f0[q]; f0[q] = f1[q]; f1[q] = f2[q];
            dm1[q] = d0[q]; d0[q] = d1;
        }
        QU_s = QU;
        m_m = m_0; m_0 = m_1;
    }
}

// ---------------------------------------------------------------------------
// The two passes of a FULL-split 2D advection (advection_2d_impl with split
// 1, no horizontal diffusion), set up for kernels that run them themselves:
// first: var -> scratch, D -> scratch thickness; second: back into var and
// D.  Implemented in advection.cu (it owns the scratch buffers).
// ---------------------------------------------------------------------------
struct Advection2DPasses {
    HPassArgs<double> pass[2];
    int dir[2];  // 1: x pass, 2: y pass
};

int getm_advection_2d_passes(getm_advection* adv, getm_grid* tgrid, getm_grid* ugrid, getm_grid* vgrid,
                             int ufirst, const double* u, const double* v, double timestep, double* D,
                             const double* DU, const double* DV, double* var, int increment,
                             Advection2DPasses* out);
