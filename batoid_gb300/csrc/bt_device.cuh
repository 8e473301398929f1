// Device-side geometry for the fused sequential trace.
//
// Every function here evaluates one piece of the reference's per-ray
// arithmetic (src/*.cpp of jmeyers314/batoid) for a descriptor staged in
// shared memory.  The reference dispatches through C++ virtual calls per ray
// and per surface; here a surface is a tagged POD record and the dispatch is a
// warp-uniform switch (all lanes of a warp work on the same stage).
//
// Numerical contract: same decision rules as the reference (root choice,
// failure tests, strict/non-strict comparisons), FP64 throughout.  Where an
// expression is rearranged (e.g. the Newton step uses the un-normalised normal
// (-dz/dx, -dz/dy, 1), which leaves dt = ((rP-r).n)/(v.n) unchanged) the
// results agree with the reference to rounding.
#pragma once
#include <stdint.h>
#include <math.h>
#include "bt_desc.h"
#include "bt_ff.cuh"

struct Prog {
    const bt_stage* stages;
    const bt_surf* surfs;
    const bt_medium* media;
    const bt_obsc* obsc;
    const double* pool;
    int nstages;
    int nmedia;
    // Per-thread cache of the combined corner values of a MODAL surface
    // (batched kernel only; null elsewhere): the block's arrays, element k
    // of thread t at mc[k * mstride + t] (interleaved across the threads),
    // the cached cell of thread t at mcell[t].
    double* mc;
    float* mcf;
    int* mcell;
    int mstride;
};

__device__ __forceinline__ Prog prog_from_blob(const unsigned char* b) {
    const bt_prog_header* h = reinterpret_cast<const bt_prog_header*>(b);
    Prog p;
    p.stages = reinterpret_cast<const bt_stage*>(b + h->off_stages);
    p.surfs = reinterpret_cast<const bt_surf*>(b + h->off_surfs);
    p.media = reinterpret_cast<const bt_medium*>(b + h->off_media);
    p.obsc = reinterpret_cast<const bt_obsc*>(b + h->off_obsc);
    p.pool = reinterpret_cast<const double*>(b + h->off_pool);
    p.nstages = h->nstages;
    p.nmedia = h->nmedia;
    p.mc = nullptr;
    p.mcf = nullptr;
    p.mcell = nullptr;
    p.mstride = 0;
    return p;
}

// ---------------------------------------------------------------------------
// Polynomials
// ---------------------------------------------------------------------------

// 1-D Horner over coefs[0..n), highest power last (src/polynomialSurface.cpp:50-57).
__device__ __forceinline__ double bt_horner(double x, const double* c, int n) {
    double r = 0.0;
    for (int i = n - 1; i >= 0; i--) r = r * x + c[i];
    return r;
}

// 2-D Horner: coefs laid out [iy][ix] (row i is the polynomial in y for x^i
// in the reference's indexing; src/polynomialSurface.cpp:59-66).
__device__ __forceinline__ double bt_horner2d(double x, double y, const double* c, int nx, int ny) {
    double r = 0.0;
    for (int i = ny - 1; i >= 0; i--) r = r * x + bt_horner(y, c + i * nx, nx);
    return r;
}

// ---------------------------------------------------------------------------
// Bicubic table (src/table.cpp:42-158)
// ---------------------------------------------------------------------------

template <typename T>
__device__ __forceinline__ T bt_spline1(T x, T v0, T v1, T d0, T d1) {
    T a = 2 * (v0 - v1) + d0 + d1;
    T b = 3 * (v1 - v0) - 2 * d0 - d1;
    return v0 + x * (d0 + x * (b + x * a));
}

template <typename T>
__device__ __forceinline__ T bt_spline1_grad(T x, T v0, T v1, T d0, T d1) {
    T a = 2 * (v0 - v1) + d0 + d1;
    T b = 3 * (v1 - v0) - 2 * d0 - d1;
    return d0 + x * (2 * b + x * 3 * a);
}

// Hermite bicubic patch from its 16 corner values; corner k of z/zx/zy/c is
// 0 = (ix, iy), 1 = (ix+1, iy), 2 = (ix, iy+1), 3 = (ix+1, iy+1)
// (src/table.cpp:64-158).
template <typename T>
__device__ __forceinline__ void bt_hermite(T xfrac, T yfrac, T dx, T dy, const T* z, const T* zx, const T* zy,
                                           const T* c, T* val, T* gx, T* gy, bool want_val, bool want_grad) {
    if (want_val) {
        T v0 = bt_spline1(xfrac, z[0], z[1], zx[0] * dx, zx[1] * dx);
        T v1 = bt_spline1(xfrac, z[2], z[3], zx[2] * dx, zx[3] * dx);
        T d0 = bt_spline1(xfrac, zy[0], zy[1], c[0] * dx, c[1] * dx);
        T d1 = bt_spline1(xfrac, zy[2], zy[3], c[2] * dx, c[3] * dx);
        *val = bt_spline1(yfrac, v0, v1, d0 * dy, d1 * dy);
    }
    if (want_grad) {
        T v0 = bt_spline1_grad(xfrac, z[0], z[1], zx[0] * dx, zx[1] * dx);
        T v1 = bt_spline1_grad(xfrac, z[2], z[3], zx[2] * dx, zx[3] * dx);
        T d0 = bt_spline1_grad(xfrac, zy[0], zy[1], c[0] * dx, c[1] * dx);
        T d1 = bt_spline1_grad(xfrac, zy[2], zy[3], c[2] * dx, c[3] * dx);
        *gx = bt_spline1(yfrac, v0, v1, d0 * dy, d1 * dy) / dx;
        v0 = bt_spline1_grad(yfrac, z[0], z[2], zy[0] * dy, zy[2] * dy);
        v1 = bt_spline1_grad(yfrac, z[1], z[3], zy[1] * dy, zy[3] * dy);
        d0 = bt_spline1_grad(yfrac, zx[0], zx[2], c[0] * dy, c[2] * dy);
        d1 = bt_spline1_grad(yfrac, zx[1], zx[3], c[1] * dy, c[3] * dy);
        *gy = bt_spline1(xfrac, v0, v1, d0 * dx, d1 * dx) / dy;
    }
}

// Cell of a table lookup; false outside the grid or for NaN input
// (src/table.cpp:42-62).
__device__ __forceinline__ bool bt_table_cell(const bt_surf& s, double x, double y, int* ix, int* iy,
                                              double* xfrac, double* yfrac) {
    const double x0 = s.p[0], y0 = s.p[1], dx = s.p[2], dy = s.p[3];
    const int nx = s.n, ny = s.m;
    const double fx = floor((x - x0) / dx);
    const double fy = floor((y - y0) / dy);
    if (!(fx >= 0.0) || !(fy >= 0.0) || fx >= (double)(nx - 1) || fy >= (double)(ny - 1)) return false;
    *ix = (int)fx;
    *iy = (int)fy;
    *xfrac = (x - (x0 + *ix * dx)) / dx;
    *yfrac = (y - (y0 + *iy * dy)) / dy;
    return true;
}

// Evaluates the Hermite bicubic patch value and gradient.  Returns false
// outside the grid (caller substitutes NaN or 0 per use_nan).
__device__ __forceinline__ bool bt_table_eval(const bt_surf& s, double x, double y,
                                              double* val, double* gx, double* gy,
                                              bool want_val, bool want_grad) {
    int ix, iy;
    double xfrac, yfrac;
    if (!bt_table_cell(s, x, y, &ix, &iy, &xfrac, &yfrac)) return false;
    const int nx = s.n, ny = s.m;
    const size_t plane = (size_t)nx * (size_t)ny;
    const double* Z = s.tab;
    const double* ZX = s.tab + plane;
    const double* ZY = s.tab + 2 * plane;
    const double* ZXY = s.tab + 3 * plane;
    const size_t i00 = (size_t)nx * iy + ix, i01 = i00 + 1;
    const size_t i10 = i00 + nx, i11 = i10 + 1;
    const double z[4] = {__ldg(Z + i00), __ldg(Z + i01), __ldg(Z + i10), __ldg(Z + i11)};
    const double zx[4] = {__ldg(ZX + i00), __ldg(ZX + i01), __ldg(ZX + i10), __ldg(ZX + i11)};
    const double zy[4] = {__ldg(ZY + i00), __ldg(ZY + i01), __ldg(ZY + i10), __ldg(ZY + i11)};
    const double c[4] = {__ldg(ZXY + i00), __ldg(ZXY + i01), __ldg(ZXY + i10), __ldg(ZXY + i11)};
    bt_hermite<double>(xfrac, yfrac, s.p[2], s.p[3], z, zx, zy, c, val, gx, gy, want_val, want_grad);
    return true;
}

// ---------------------------------------------------------------------------
// Sag and slope of one non-Sum surface.
//
// "slope" returns (ux, uy) = (nx/nz, ny/nz) of the reference's unit normal,
// i.e. the un-normalised normal is (ux, uy, 1).  For every kind except Tilted
// this is (-dz/dx, -dz/dy); Tilted reproduces the reference's own normal
// (-tanx, -tany, sqrt(1-tanx^2-tany^2)) (src/tilted.cpp:20-27).
// ---------------------------------------------------------------------------

__device__ __forceinline__ void bt_leaf_eval(const bt_surf& s, const double* pool,
                                             double x, double y,
                                             bool want_sag, bool want_slope,
                                             double* sag, double* ux, double* uy) {
    switch (s.kind) {
    case BT_S_PLANE:
        if (want_sag) *sag = 0.0;
        if (want_slope) { *ux = 0.0; *uy = 0.0; }
        break;
    case BT_S_TILTED:
        if (want_sag) *sag = x * s.p[0] + y * s.p[1];
        if (want_slope) { *ux = -s.p[0] / s.p[2]; *uy = -s.p[1] / s.p[2]; }
        break;
    case BT_S_SPHERE: {
        // src/sphere.cpp:15-48
        const double R = s.p[0];
        if (R == 0.0) {
            if (want_sag) *sag = 0.0;
            if (want_slope) { *ux = 0.0; *uy = 0.0; }
            break;
        }
        const double r2 = x * x + y * y;
        if (want_sag) *sag = R * (1 - sqrt(1 - r2 * s.p[3]));
        if (want_slope) {
            // (dz/dr)/r = (1/R) / sqrt(1 - (r/R)^2)
            const double k = s.p[2] / sqrt(1 - r2 * s.p[3]);
            *ux = -x * k;
            *uy = -y * k;
        }
        break;
    }
    case BT_S_PARABOLOID: {
        // src/paraboloid.cpp:15-37
        if (s.p[0] == 0.0) {
            if (want_sag) *sag = 0.0;
            if (want_slope) { *ux = 0.0; *uy = 0.0; }
            break;
        }
        if (want_sag) *sag = (x * x + y * y) * s.p[2];
        if (want_slope) { *ux = -x * s.p[1]; *uy = -y * s.p[1]; }
        break;
    }
    case BT_S_QUADRIC:
    case BT_S_ASPHERE: {
        // src/quadric.cpp:18-38, src/asphere.cpp:37-74
        const double R = s.p[0];
        const double r2 = x * x + y * y;
        double z = 0.0, k = 0.0;
        if (R != 0.0) {
            const double q = sqrt(1. - r2 * s.p[8]);
            if (want_sag) z = r2 / (R * (1. + q));
            if (want_slope) k = 1.0 / (R * q);   // (dz/dr)/r of the conic
        }
        if (s.kind == BT_S_ASPHERE) {
            const double* c = pool + s.off;
            const double* dc = c + s.n;
            // sum_i c_i r^(2i+2) and sum_i dc_i r^(2i) by Horner in r^2
            double a = 0.0, da = 0.0;
            for (int i = s.n - 1; i >= 0; i--) {
                a = a * r2 + c[i];
                da = da * r2 + dc[i];
            }
            z += a * r2;
            k += da;
        }
        if (want_sag) *sag = z;
        if (want_slope) { *ux = -x * k; *uy = -y * k; }
        break;
    }
    case BT_S_POLY: {
        // src/polynomialSurface.cpp:35-48
        const double xx = x - s.p[0], yy = y - s.p[1];
        const double* c = pool + s.off;
        const int nx = s.n, ny = s.m;
        if (want_sag) *sag = bt_horner2d(xx, yy, c, nx, ny);
        if (want_slope) {
            const int gsz = (nx - 1) * (ny - 1);
            const double* gxc = c + nx * ny;
            const double* gyc = gxc + gsz;
            *ux = -bt_horner2d(xx, yy, gxc, nx - 1, ny - 1);
            *uy = -bt_horner2d(xx, yy, gyc, nx - 1, ny - 1);
        }
        break;
    }
    case BT_S_BICUBIC: {
        // src/bicubic.cpp:19-40
        double v = 0.0, gx = 0.0, gy = 0.0;
        bool inside = bt_table_eval(s, x, y, &v, &gx, &gy, want_sag, want_slope);
        if (!inside) {
            const double fill = (s.p[4] != 0.0) ? (double)NAN : 0.0;
            v = fill; gx = fill; gy = fill;
        }
        if (want_sag) *sag = v;
        if (want_slope) { *ux = -gx; *uy = -gy; }
        break;
    }
    default:
        if (want_sag) *sag = NAN;
        if (want_slope) { *ux = NAN; *uy = NAN; }
        break;
    }
}

// ---------------------------------------------------------------------------
// MODAL surface: sum_m a_m * table_m over bicubic tables sharing one grid.
// The Hermite patch is linear in its 16 corner values, so the patch of the
// weighted sum is the patch of the weighted corner values.  Those are formed
// once per (ray, cell) in float-float (FP32 mode data, amplitudes as
// float-float pairs, ~44-bit sums) and cached per thread; Newton iterates of
// one ray nearly always stay in one cell.  The cache is invalidated (cell
// -1) whenever the amplitudes change.
// ---------------------------------------------------------------------------

// a * b for float-float a and float b; the pair is left unnormalised (the
// following ff_add renormalises).
__device__ __forceinline__ ff ff_mulf(ff a, float b) {
    const float p = a.hi * b;
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return ff{p, e};
}

// Cell lookup with the reciprocal grid steps p[6] = 1/dx, p[7] = 1/dy
// (no division).  Where rounding moves a point across a cell edge the
// neighbouring patch gives the same value and slope to rounding: Hermite
// patches are C1 across edges.
__device__ __forceinline__ bool bt_modal_cell(const bt_surf& s, double x, double y, int* ix, int* iy,
                                              double* xfrac, double* yfrac) {
    const double x0 = s.p[0], y0 = s.p[1], dx = s.p[2], dy = s.p[3];
    const double fx = floor((x - x0) * s.p[6]);
    const double fy = floor((y - y0) * s.p[7]);
    if (!(fx >= 0.0) || !(fy >= 0.0) || fx >= (double)(s.n - 1) || fy >= (double)(s.m - 1)) return false;
    *ix = (int)fx;
    *iy = (int)fy;
    *xfrac = (x - (x0 + *ix * dx)) * s.p[6];
    *yfrac = (y - (y0 + *iy * dy)) * s.p[7];
    return true;
}

// Weighted corner values of cell (ix, iy) into the per-thread cache; out of
// line: it runs once per ray and cell, the Newton iterations that use the
// cache are the hot path.
static __device__ __noinline__ void bt_modal_fill(const double* pool, const bt_surf* sp, int ix, int iy, double* mc,
                                           float* mcf, int st) {
    const bt_surf& s = *sp;
    const int nx = s.n;
    const int nq = (int)s.p[5] / 4;  // float4 groups per quantity
    const ff* a = ff_ptr(pool, s.off);
    const float4* T = reinterpret_cast<const float4*>(s.tab);
    const size_t node0 = (size_t)nx * iy + ix;
    for (int c = 0; c < 4; c++) {
        const size_t node = node0 + (c & 1) + ((c >> 1) ? (size_t)nx : 0);
        const float4* v = T + node * (size_t)(4 * nq);
        for (int q = 0; q < 4; q++) {
            ff acc{0.f, 0.f};
            for (int k = 0; k < nq; k++) {
                const float4 w = __ldg(v + q * nq + k);
                acc = ff_add(acc, ff_mulf(a[4 * k + 0], w.x));
                acc = ff_add(acc, ff_mulf(a[4 * k + 1], w.y));
                acc = ff_add(acc, ff_mulf(a[4 * k + 2], w.z));
                acc = ff_add(acc, ff_mulf(a[4 * k + 3], w.w));
            }
            mc[(q * 4 + c) * st] = ff_to_double(acc);
            mcf[(q * 4 + c) * st] = acc.hi + acc.lo;
        }
    }
}

__device__ __forceinline__ bool bt_modal_locate(const Prog& P, const bt_surf& s, double x, double y,
                                                double* xfrac, double* yfrac) {
    int ix, iy;
    if (!bt_modal_cell(s, x, y, &ix, &iy, xfrac, yfrac)) return false;
    const int cell = iy * s.n + ix;
    int* cellp = P.mcell + threadIdx.x;
    if (*cellp == cell) return true;
    bt_modal_fill(P.pool, &s, ix, iy, P.mc + threadIdx.x, P.mcf + threadIdx.x, P.mstride);
    *cellp = cell;
    return true;
}

// FP64 sag and slope (ux, uy) = (-dz/dx, -dz/dy) (src/bicubic.cpp:19-40).
__device__ __forceinline__ void bt_modal_eval(const Prog& P, const bt_surf& s, double x, double y,
                                              bool want_sag, bool want_slope, double* sag, double* ux,
                                              double* uy) {
    double xf, yf;
    if (P.mc == nullptr || !bt_modal_locate(P, s, x, y, &xf, &yf)) {
        const double fill = (P.mc == nullptr || s.p[4] != 0.0) ? (double)NAN : 0.0;
        if (want_sag) *sag = fill;
        if (want_slope) { *ux = fill; *uy = fill; }
        return;
    }
    const int st = P.mstride;
    double v[16];
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = P.mc[k * st + threadIdx.x];
    double val = 0.0, gx = 0.0, gy = 0.0;
    bt_hermite<double>(xf, yf, s.p[2], s.p[3], v, v + 4, v + 8, v + 12, &val, &gx, &gy, want_sag, want_slope);
    if (want_sag) *sag = val;
    if (want_slope) { *ux = -gx; *uy = -gy; }
}

// FP64 sag with an FP32 slope, for Newton iterations.
__device__ __forceinline__ void bt_modal_newton_eval(const Prog& P, const bt_surf& s, double x, double y,
                                                     double* sag, float* ux, float* uy) {
    double xf, yf;
    if (P.mc == nullptr || !bt_modal_locate(P, s, x, y, &xf, &yf)) {
        const double fill = (P.mc == nullptr || s.p[4] != 0.0) ? (double)NAN : 0.0;
        *sag = fill;
        *ux = (float)fill;
        *uy = (float)fill;
        return;
    }
    const int st = P.mstride;
    double v[16];
    float w[16];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        v[k] = P.mc[k * st + threadIdx.x];
        w[k] = P.mcf[k * st + threadIdx.x];
    }
    double val;
    bt_hermite<double>(xf, yf, s.p[2], s.p[3], v, v + 4, v + 8, v + 12, &val, nullptr, nullptr, true, false);
    float gx, gy;
    bt_hermite<float>((float)xf, (float)yf, (float)s.p[2], (float)s.p[3], w, w + 4, w + 8, w + 12, nullptr, &gx,
                      &gy, false, true);
    *sag = val;
    *ux = -gx;
    *uy = -gy;
}

// Sag and slope of any surface (Sum adds its children: src/sum.cpp:23-45).
__device__ __forceinline__ void bt_surf_eval(const Prog& P, int si, double x, double y,
                                             bool want_sag, bool want_slope,
                                             double* sag, double* ux, double* uy) {
    const bt_surf& s = P.surfs[si];
    if (s.kind == BT_S_MODAL) {
        bt_modal_eval(P, s, x, y, want_sag, want_slope, sag, ux, uy);
        return;
    }
    if (s.kind != BT_S_SUM) {
        bt_leaf_eval(s, P.pool, x, y, want_sag, want_slope, sag, ux, uy);
        return;
    }
    double z = 0.0, gx = 0.0, gy = 0.0;
    for (int c = 0; c < s.n; c++) {
        double cz = 0.0, cx = 0.0, cy = 0.0;
        const bt_surf& cs = P.surfs[s.m + c];
        if (cs.kind == BT_S_MODAL) bt_modal_eval(P, cs, x, y, want_sag, want_slope, &cz, &cx, &cy);
        else bt_leaf_eval(cs, P.pool, x, y, want_sag, want_slope, &cz, &cx, &cy);
        z += cz; gx += cx; gy += cy;
    }
    if (want_sag) *sag = z;
    if (want_slope) { *ux = gx; *uy = gy; }
}

// ---------------------------------------------------------------------------
// Intersections
// ---------------------------------------------------------------------------

// Newton / tangent-plane iteration of the reference (src/surface.cpp:22-49).
// Stops early once an iterate reproduces the previous one exactly: the
// iteration map is a pure function of dt, so every further iteration would
// return the same state and the converged result is identical to running all
// `niter` iterations.  On exit (ux, uy) hold the slope at the final point.
__device__ __forceinline__ bool bt_newton(const Prog& P, int si,
                                          double x, double y, double z,
                                          double vx, double vy, double vz,
                                          double& dt, int niter,
                                          double* ux, double* uy) {
    double rPx = x + vx * dt;
    double rPy = y + vy * dt;
    double rPz = z + vz * dt;
    double sz, gx, gy;
    bt_surf_eval(P, si, rPx, rPy, true, true, &sz, &gx, &gy);
    for (int it = 0; it < niter; it++) {
        // dt = ((rP - r).n) / (v.n) with n ~ (gx, gy, 1)
        double num = (rPx - x) * gx + (rPy - y) * gy + (sz - z);
        double den = gx * vx + gy * vy + vz;
        double dtn = num / den;
        if (dtn == dt) break;
        dt = dtn;
        rPx = x + vx * dt;
        rPy = y + vy * dt;
        rPz = z + vz * dt;
        bt_surf_eval(P, si, rPx, rPy, true, true, &sz, &gx, &gy);
    }
    *ux = gx;
    *uy = gy;
    return fabs(sz - rPz) < 1e-12;
}

// Stable quadratic root pair of the reference (src/sphere.cpp:51-58 and
// siblings).  Returns false for a negative discriminant.
__device__ __forceinline__ bool bt_quad_roots(double a, double b, double c, double* dt1, double* dt2) {
    double disc = b * b - 4 * a * c;
    if (disc < 0) return false;
    double r1;
    if (b > 0) r1 = (-b - sqrt(disc)) / (2 * a);
    else r1 = 2 * c / (-b + sqrt(disc));
    *dt1 = r1;
    *dt2 = c / (a * r1);
    return true;
}

// Analytic or iterative time-to-intersect of a non-Sum surface.  `slope_ok`
// is set when (ux, uy) already hold the slope at the intersection.
__device__ __forceinline__ bool bt_leaf_tti(const Prog& P, int si,
                                            double x, double y, double z,
                                            double vx, double vy, double vz,
                                            double& dt, int niter,
                                            double* ux, double* uy, bool* slope_ok) {
    const bt_surf& s = P.surfs[si];
    *slope_ok = false;
    switch (s.kind) {
    case BT_S_PLANE:
        // src/plane.cpp:23-30
        if (vz == 0) return false;
        dt = -z / vz;
        return true;
    case BT_S_TILTED: {
        // src/tilted.cpp:29-37
        double num = z - x * s.p[0] - y * s.p[1];
        double den = vx * s.p[0] + vy * s.p[1] - vz;
        if (den == 0) return false;
        dt = num / den;
        return true;
    }
    case BT_S_SPHERE: {
        // src/sphere.cpp:36-67
        const double R = s.p[0];
        double vr2 = vx * vx + vy * vy;
        double vz2 = vz * vz;
        double vrr0 = vx * x + vy * y;
        double r02 = x * x + y * y;
        double z0 = z - R;
        double a = vz2 + vr2;
        double b = 2 * vz * z0 + 2 * vrr0;
        double c = z0 * z0 - s.p[1] + r02;
        double t1, t2;
        if (!bt_quad_roots(a, b, c, &t1, &t2)) return false;
        dt = (vz * R < 0) ? fmax(t1, t2) : fmin(t1, t2);
        return true;
    }
    case BT_S_PARABOLOID: {
        // src/paraboloid.cpp:38-71
        double a = (vx * vx + vy * vy) * s.p[2];
        double b = (x * vx + y * vy) * s.p[1] - vz;
        double c = (x * x + y * y) * s.p[2] - z;
        if (a == 0) { dt = -c / b; return true; }
        double t1, t2;
        if (!bt_quad_roots(a, b, c, &t1, &t2)) return false;
        dt = (vz * s.p[0] < 0) ? fmax(t1, t2) : fmin(t1, t2);
        return true;
    }
    case BT_S_QUADRIC:
    case BT_S_ASPHERE: {
        // src/quadric.cpp:41-71; Asphere starts Newton from it (src/asphere.cpp:76-85)
        double z0 = z - s.p[6];
        double vrr0 = vx * x + vy * y;
        double a = vz * vz + (vx * vx + vy * vy) * s.p[5];
        double b = 2 * (vz * z0 + vrr0 * s.p[5]);
        double c = z0 * z0 - s.p[7] + (x * x + y * y) * s.p[5];
        double t1, t2;
        if (!bt_quad_roots(a, b, c, &t1, &t2)) return false;
        double z1 = z + vz * t1;
        double z2 = z + vz * t2;
        dt = (fabs(z1) < fabs(z2)) ? t1 : t2;
        if (s.kind == BT_S_QUADRIC) return true;
        *slope_ok = true;
        return bt_newton(P, si, x, y, z, vx, vy, vz, dt, niter, ux, uy);
    }
    default:
        // PolynomialSurface, Bicubic: generic Newton from the given dt
        *slope_ok = true;
        return bt_newton(P, si, x, y, z, vx, vy, vz, dt, niter, ux, uy);
    }
}

__device__ __forceinline__ bool bt_surf_tti(const Prog& P, int si,
                                            double x, double y, double z,
                                            double vx, double vy, double vz,
                                            double& dt, int niter,
                                            double* ux, double* uy, bool* slope_ok) {
    const bt_surf& s = P.surfs[si];
    if (s.kind != BT_S_SUM)
        return bt_leaf_tti(P, si, x, y, z, vx, vy, vz, dt, niter, ux, uy, slope_ok);
    // Sum: first child's own solve as the starting point, then Newton on the
    // sum (src/sum.cpp:47-56).
    bool dummy;
    if (!bt_leaf_tti(P, s.m, x, y, z, vx, vy, vz, dt, niter, ux, uy, &dummy)) return false;
    *slope_ok = true;
    return bt_newton(P, si, x, y, z, vx, vy, vz, dt, niter, ux, uy);
}

// Unit normal at (x, y) from the slope form.
__device__ __forceinline__ void bt_normal_from_slope(double ux, double uy, double* nx, double* ny, double* nz) {
    double k = 1.0 / sqrt(ux * ux + uy * uy + 1.0);
    *nx = ux * k;
    *ny = uy * k;
    *nz = k;
}

// The reference's exact normal for surfaces where the slope form and the
// reference's expression agree only in exact arithmetic, evaluated fresh.
__device__ __forceinline__ void bt_surf_normal(const Prog& P, int si, double x, double y,
                                               double* nx, double* ny, double* nz) {
    const bt_surf& s = P.surfs[si];
    if (s.kind == BT_S_TILTED) {
        *nx = -s.p[0]; *ny = -s.p[1]; *nz = s.p[2];
        return;
    }
    if (s.kind == BT_S_PLANE) { *nx = 0.0; *ny = 0.0; *nz = 1.0; return; }
    double ux, uy, dummy;
    bt_surf_eval(P, si, x, y, false, true, &dummy, &ux, &uy);
    bt_normal_from_slope(ux, uy, nx, ny, nz);
}

// ---------------------------------------------------------------------------
// Media (src/medium.cpp)
// ---------------------------------------------------------------------------

__device__ __forceinline__ double bt_getN(const Prog& P, int mi, double w) {
    const bt_medium& m = P.media[mi];
    switch (m.kind) {
    case BT_M_CONST:
        return m.p[0];
    case BT_M_TABLE: {
        // linear search + interpolation, NaN outside (src/medium.cpp:89-105)
        const double* args = P.pool + m.off;
        const double* vals = args + m.n;
        if (w < args[0]) return NAN;
        if (w > args[m.n - 1]) return NAN;
        if (m.n < 2) return vals[0];  // single entry and w == args[0]
        int u;
        for (u = 1; u < m.n; u++)
            if (w < args[u]) break;
        if (u >= m.n) u = m.n - 1;  // w == last arg
        double out = (w - args[u - 1]);
        out *= (vals[u] - vals[u - 1]);
        out /= (args[u] - args[u - 1]);
        out += vals[u - 1];
        return out;
    }
    case BT_M_SELLMEIER: {
        // src/medium.cpp:145-149, wavelength in microns squared
        double x = w * w * 1e12;
        return sqrt(1.0 + m.p[0] * x / (x - m.p[3]) + m.p[1] * x / (x - m.p[4]) + m.p[2] * x / (x - m.p[5]));
    }
    case BT_M_SUMITA: {
        // src/medium.cpp:186-191
        double x = w * w * 1e12;
        double y = 1. / x;
        return sqrt(m.p[0] + m.p[1] * x + y * (m.p[2] + y * (m.p[3] + y * (m.p[4] + y * m.p[5]))));
    }
    case BT_M_AIR: {
        // Edlen / Filippenko (src/medium.cpp:237-245)
        const double P_ = m.p[0], T = m.p[1], W = m.p[2];
        double s2 = 1e-12 / (w * w);
        double nm1 = (64.328 + (29498.1 / (146.0 - s2)) + (255.4 / (41.0 - s2))) * 1.e-6;
        nm1 *= P_ * (1.0 + (1.049 - 0.0157 * T) * 1.e-6 * P_) / (720.883 * (1.0 + 0.003661 * T));
        nm1 -= (0.0624 - 0.000680 * s2) / (1.0 + 0.003661 * T) * W * 1.e-6;
        return 1 + nm1;
    }
    default:
        return NAN;
    }
}

// ---------------------------------------------------------------------------
// Obscurations (src/obscuration.cpp), evaluated as a postfix program.
// ---------------------------------------------------------------------------

__device__ __forceinline__ bool bt_polygon_contains(const double* xp, const double* yp, int n, double x, double y) {
    // even-odd crossing test (src/obscuration.cpp:201-225)
    double x1 = xp[0], y1 = yp[0];
    double xinters = 0.0;
    bool inside = false;
    for (int i = 1; i <= n; i++) {
        int k = (i == n) ? 0 : i;
        double x2 = xp[k], y2 = yp[k];
        if (y > fmin(y1, y2)) {
            if (y <= fmax(y1, y2)) {
                if (x <= fmax(x1, x2)) {
                    if (y1 != y2) xinters = (y - y1) * (x2 - x1) / (y2 - y1) + x1;
                    if (x1 == x2 || x <= xinters) inside = !inside;
                }
            }
        }
        x1 = x2;
        y1 = y2;
    }
    return inside;
}

// hypot(dx, dy) < r (the reference's test, src/obscuration.cpp:32-34, 80-83),
// decided from dx^2 + dy^2 vs r^2 unless the two are within a relative
// 1e-13 of each other, where hypot itself decides.
__device__ __forceinline__ bool bt_radius_less(double dx, double dy, double r, bool) {
    const double h2 = dx * dx + dy * dy;
    const double r2 = r * r;
    if (h2 < r2 * (1.0 - 1e-13)) return r > 0.0;
    if (h2 > r2 * (1.0 + 1e-13)) return false;
    return hypot(dx, dy) < r;
}

__device__ __forceinline__ bool bt_obsc_run(const Prog& P, int begin, int end, double x, double y) {
    uint32_t stack = 0;  // bit k = entry k
    int sp = 0;
    for (int k = begin; k < end; k++) {
        const bt_obsc& o = P.obsc[k];
        bool v = false;
        switch (o.op) {
        case BT_O_CIRCLE:
            v = bt_radius_less(x - o.p[1], y - o.p[2], o.p[0], false);
            break;
        case BT_O_ANNULUS: {
            const double dx = x - o.p[2], dy = y - o.p[3];
            v = !bt_radius_less(dx, dy, o.p[0], false) && bt_radius_less(dx, dy, o.p[1], false);
            break;
        }
        case BT_O_RECT: {
            double xp = (x - o.p[2]) * o.p[5] + (y - o.p[3]) * o.p[4];
            double yp = -(x - o.p[2]) * o.p[4] + (y - o.p[3]) * o.p[5];
            v = (xp > -o.p[0] / 2 && xp < o.p[0] / 2 && yp > -o.p[1] / 2 && yp < o.p[1] / 2);
            break;
        }
        case BT_O_RAY: {
            double xp = (x - o.p[1]) * o.p[4] + (y - o.p[2]) * o.p[3];
            double yp = -(x - o.p[1]) * o.p[3] + (y - o.p[2]) * o.p[4];
            v = (xp > 0.0 && yp > -o.p[0] / 2 && yp < o.p[0] / 2);
            break;
        }
        case BT_O_POLYGON:
            v = bt_polygon_contains(P.pool + o.off, P.pool + o.off + o.n, o.n, x, y);
            break;
        case BT_O_NEGATION:
            sp--;
            v = !((stack >> sp) & 1u);
            break;
        case BT_O_UNION: {
            bool acc = false;
            for (int j = 0; j < o.n; j++) { sp--; acc |= (bool)((stack >> sp) & 1u); }
            v = acc;
            break;
        }
        case BT_O_INTERSECTION: {
            bool acc = true;
            for (int j = 0; j < o.n; j++) { sp--; acc &= (bool)((stack >> sp) & 1u); }
            v = acc;
            break;
        }
        default:
            break;
        }
        stack = (stack & ~(1u << sp)) | ((uint32_t)v << sp);
        sp++;
    }
    return sp > 0 ? (bool)((stack >> (sp - 1)) & 1u) : false;
}

// ===========================================================================
// Trace-kernel evaluation (mixed precision).
//
// Newton needs the residual F = sag(x + vx dt, y + vy dt) - (z + vz dt) to
// FP64 accuracy, but its derivative only approximately: with a derivative of
// relative error d, each step shrinks the error by ~d, so an FP32 slope
// (d ~ 1e-7) converges in the same 2-3 steps as the exact one.  So:
//  * sags: conic part in FP64 (one rsqrt, no division where that is exact
//    enough), polynomial perturbations (asphere terms, Zernike / Cartesian
//    polynomials) in float-float on the FP32 pipe;
//  * Newton slopes: FP32;
//  * the normal used for reflection / refraction: FP64 conic slope plus
//    float-float polynomial slope.
// Pool layout (host packer): ASPHERE [c n][dc n][c ff n][dc ff n];
// POLY [coefs][gx][gy] in FP64 then the same three arrays as float-float.
// p[9] = 1/R (0 when R == 0); p[10] = 1 when the conic sag may use
// (1 - q) * R/(1+k), i.e. |R/(1+k)| <= 100 (absolute error <= 100 ulp(1)).
// ===========================================================================

// sqrt(w) from w * rsqrt(w), exact for w == 0 and NaN for w < 0.
__device__ __forceinline__ void bt_sqrt_rsqrt(double w, double* q, double* rs) {
    if (w > 0.0) {
        const double r = rsqrt(w);
        *rs = r;
        *q = w * r;
    } else {
        *q = sqrt(w);
        *rs = 1.0 / *q;
    }
}

// Conic of a QUADRIC / ASPHERE record: sag and (dz/dr)/r, FP64.
__device__ __forceinline__ void bt_conic(const bt_surf& s, double r2, double* sag, double* k) {
    if (s.p[0] == 0.0) {
        *sag = 0.0;
        *k = 0.0;
        return;
    }
    const double w = 1. - r2 * s.p[8];
    double q, rs;
    bt_sqrt_rsqrt(w, &q, &rs);
    *sag = (s.p[10] != 0.0) ? (1. - q) * s.p[6] : r2 / (s.p[0] * (1. + q));
    *k = rs * s.p[9];
}

__device__ __forceinline__ void bt_sphere_conic(const bt_surf& s, double r2, double* sag, double* k) {
    if (s.p[0] == 0.0) {
        *sag = 0.0;
        *k = 0.0;
        return;
    }
    const double w = 1. - r2 * s.p[3];
    double q, rs;
    bt_sqrt_rsqrt(w, &q, &rs);
    *sag = s.p[0] * (1. - q);
    *k = rs * s.p[2];
}

// FP64-accurate sag with an FP32 slope (Newton iterations).
__device__ __forceinline__ void bt_leaf_newton_eval(const bt_surf& s, const double* pool, double x, double y,
                                                    double* sag, float* ux, float* uy) {
    switch (s.kind) {
    case BT_S_PLANE:
        *sag = 0.0; *ux = 0.f; *uy = 0.f;
        return;
    case BT_S_TILTED:
        *sag = x * s.p[0] + y * s.p[1];
        *ux = (float)(-s.p[0] / s.p[2]);
        *uy = (float)(-s.p[1] / s.p[2]);
        return;
    case BT_S_SPHERE: {
        double k;
        bt_sphere_conic(s, x * x + y * y, sag, &k);
        *ux = (float)(-x * k);
        *uy = (float)(-y * k);
        return;
    }
    case BT_S_PARABOLOID:
        if (s.p[0] == 0.0) { *sag = 0.0; *ux = 0.f; *uy = 0.f; return; }
        *sag = (x * x + y * y) * s.p[2];
        *ux = (float)(-x * s.p[1]);
        *uy = (float)(-y * s.p[1]);
        return;
    case BT_S_QUADRIC:
    case BT_S_ASPHERE: {
        const double r2 = x * x + y * y;
        double z, k;
        bt_conic(s, r2, &z, &k);
        float kf = (float)k;
        if (s.kind == BT_S_ASPHERE && s.n > 0) {
            const ff r2f = ff_from(r2);
            const ff* c = ff_ptr(pool, s.off + 2 * s.n);
            const ff* dc = c + s.n;
            const ff a = ff_mul(ff_horner(r2f, c, s.n), r2f);
            z += ff_to_double(a);
            float da = 0.f;
            for (int i = s.n - 1; i >= 0; i--) da = fmaf(da, r2f.hi, dc[i].hi);
            kf += da;
        }
        *sag = z;
        *ux = (float)(-x) * kf;
        *uy = (float)(-y) * kf;
        return;
    }
    case BT_S_POLY: {
        const double xx = x - s.p[0], yy = y - s.p[1];
        const int nx = s.n, ny = s.m;
        const int g = (nx - 1) * (ny - 1);
        const ff* c = ff_ptr(pool, s.off + nx * ny + 2 * g);
        *sag = ff_to_double(ff_horner2d(ff_from(xx), ff_from(yy), c, nx, ny));
        const float fx = (float)xx, fy = (float)yy;
        *ux = -f_horner2d(fx, fy, c + nx * ny, nx - 1, ny - 1);
        *uy = -f_horner2d(fx, fy, c + nx * ny + g, nx - 1, ny - 1);
        return;
    }
    default: {
        double z, gx, gy;
        bt_leaf_eval(s, pool, x, y, true, true, &z, &gx, &gy);
        *sag = z;
        *ux = (float)gx;
        *uy = (float)gy;
        return;
    }
    }
}

__device__ __forceinline__ void bt_surf_newton_eval(const Prog& P, int si, double x, double y, double* sag,
                                                    float* ux, float* uy) {
    const bt_surf& s = P.surfs[si];
    if (s.kind == BT_S_MODAL) {
        bt_modal_newton_eval(P, s, x, y, sag, ux, uy);
        return;
    }
    if (s.kind != BT_S_SUM) {
        bt_leaf_newton_eval(s, P.pool, x, y, sag, ux, uy);
        return;
    }
    double z = 0.0;
    float gx = 0.f, gy = 0.f;
    for (int c = 0; c < s.n; c++) {
        double cz;
        float cx, cy;
        const bt_surf& cs = P.surfs[s.m + c];
        if (cs.kind == BT_S_MODAL) bt_modal_newton_eval(P, cs, x, y, &cz, &cx, &cy);
        else bt_leaf_newton_eval(cs, P.pool, x, y, &cz, &cx, &cy);
        z += cz;
        gx += cx;
        gy += cy;
    }
    *sag = z;
    *ux = gx;
    *uy = gy;
}

// Slope (nx/nz, ny/nz) at full accuracy for the interaction normal.
__device__ __forceinline__ void bt_leaf_slope_precise(const bt_surf& s, const double* pool, double x, double y,
                                                      double* ux, double* uy) {
    switch (s.kind) {
    case BT_S_SPHERE: {
        double z, k;
        bt_sphere_conic(s, x * x + y * y, &z, &k);
        *ux = -x * k;
        *uy = -y * k;
        return;
    }
    case BT_S_QUADRIC:
    case BT_S_ASPHERE: {
        const double r2 = x * x + y * y;
        double z, k;
        bt_conic(s, r2, &z, &k);
        if (s.kind == BT_S_ASPHERE && s.n > 0) {
            const ff* dc = ff_ptr(pool, s.off + 3 * s.n);
            k += ff_to_double(ff_horner(ff_from(r2), dc, s.n));
        }
        *ux = -x * k;
        *uy = -y * k;
        return;
    }
    case BT_S_POLY: {
        const int nx = s.n, ny = s.m;
        const int g = (nx - 1) * (ny - 1);
        const ff* c = ff_ptr(pool, s.off + nx * ny + 2 * g);
        const ff xf = ff_from(x - s.p[0]), yf = ff_from(y - s.p[1]);
        *ux = -ff_to_double(ff_horner2d(xf, yf, c + nx * ny, nx - 1, ny - 1));
        *uy = -ff_to_double(ff_horner2d(xf, yf, c + nx * ny + g, nx - 1, ny - 1));
        return;
    }
    default: {
        double z;
        bt_leaf_eval(s, pool, x, y, false, true, &z, ux, uy);
        return;
    }
    }
}

__device__ __forceinline__ void bt_surf_slope_precise(const Prog& P, int si, double x, double y, double* ux,
                                                      double* uy) {
    const bt_surf& s = P.surfs[si];
    double z;
    if (s.kind == BT_S_MODAL) {
        bt_modal_eval(P, s, x, y, false, true, &z, ux, uy);
        return;
    }
    if (s.kind != BT_S_SUM) {
        bt_leaf_slope_precise(s, P.pool, x, y, ux, uy);
        return;
    }
    double gx = 0.0, gy = 0.0;
    for (int c = 0; c < s.n; c++) {
        double cx, cy;
        const bt_surf& cs = P.surfs[s.m + c];
        if (cs.kind == BT_S_MODAL) bt_modal_eval(P, cs, x, y, false, true, &z, &cx, &cy);
        else bt_leaf_slope_precise(cs, P.pool, x, y, &cx, &cy);
        gx += cx;
        gy += cy;
    }
    *ux = gx;
    *uy = gy;
}

// Unit normal at the intersection (reference conventions, incl. Tilted).
__device__ __forceinline__ void bt_normal_precise(const Prog& P, int si, double x, double y, double* nx,
                                                  double* ny, double* nz) {
    const bt_surf& s = P.surfs[si];
    if (s.kind == BT_S_TILTED) { *nx = -s.p[0]; *ny = -s.p[1]; *nz = s.p[2]; return; }
    if (s.kind == BT_S_PLANE) { *nx = 0.0; *ny = 0.0; *nz = 1.0; return; }
    if (s.kind == BT_S_SPHERE && s.p[0] != 0.0) {
        // (-x k, -y k, 1) / |.| with k = 1/(R q), q = sqrt(1 - r^2/R^2): the
        // norm is 1/q, so the unit normal is (-x/R, -y/R, q)
        double q, rs;
        bt_sqrt_rsqrt(1. - (x * x + y * y) * s.p[3], &q, &rs);
        *nx = -x * s.p[2];
        *ny = -y * s.p[2];
        *nz = q;
        return;
    }
    double ux, uy;
    bt_surf_slope_precise(P, si, x, y, &ux, &uy);
    const double k = rsqrt(ux * ux + uy * uy + 1.0);
    *nx = ux * k;
    *ny = uy * k;
    *nz = k;
}

// Newton in correction form: dt += F / F'(approx).  Stops at an exact fixed
// point, or once a correction below 1e-11 has been applied and the surface
// re-evaluated there (the next correction would be < 1e-11 times the FP32
// derivative's relative error), or after niter steps as the reference.
// The reference's success test is |F| < 1e-12 at the final point.  When a
// correction below 1e-11 is applied to a point whose |F| is already below
// 1e-12, the residual there is |F| times the derivative's relative error
// (~1e-7), so the test passes without evaluating the surface again: the
// returned dt is the same, one sag evaluation is saved.
__device__ __forceinline__ bool bt_newton_mixed(const Prog& P, int si, double x, double y, double z, double vx,
                                                double vy, double vz, double& dt, int niter) {
    double rPx = x + vx * dt;
    double rPy = y + vy * dt;
    double rPz = z + vz * dt;
    double sz;
    float gx, gy;
    bt_surf_newton_eval(P, si, rPx, rPy, &sz, &gx, &gy);
    double res = sz - rPz;
    const float fvx = (float)vx, fvy = (float)vy, fvz = (float)vz;
    for (int it = 0; it < niter; it++) {
        const float den = fmaf(gx, fvx, fmaf(gy, fvy, fvz));
        const double ddt = res * (double)(1.0f / den);
        const double dtn = dt + ddt;
        if (dtn == dt) break;
        dt = dtn;
        const bool small = fabs(ddt) < 1e-11;
        if (small && fabs(res) < 1e-12) return true;
        rPx = x + vx * dt;
        rPy = y + vy * dt;
        rPz = z + vz * dt;
        bt_surf_newton_eval(P, si, rPx, rPy, &sz, &gx, &gy);
        res = sz - rPz;
        if (small) break;
    }
    return fabs(res) < 1e-12;
}

// One root of a*t^2 + b*t + c = 0 with one division: `plus` selects
// (-b + sqrt(D)) / 2a, else (-b - sqrt(D)) / 2a; each in its cancellation-
// free form (the reference's dt1 / dt2 pair, src/sphere.cpp:51-58).
__device__ __forceinline__ bool bt_one_root(double a, double b, double c, bool plus, double* t) {
    const double disc = b * b - 4 * a * c;
    if (disc < 0) return false;
    double s, rs;
    bt_sqrt_rsqrt(disc, &s, &rs);
    if (b > 0) *t = plus ? 2 * c / (-b - s) : (-b - s) / (2 * a);
    else *t = plus ? (-b + s) / (2 * a) : 2 * c / (-b + s);
    return true;
}

// One Newton step in FP32 from an asphere's conic root.  There the conic
// part of the sag equals z up to FP64 rounding, so the residual is the
// polynomial part alone, which FP32 evaluates to ~1e-7 of itself (~1e-11 m
// for a 1e-4 m term); the step leaves dt ~1e-9 m from the root, where the
// FP64 Newton would arrive only after its first correction, and so saves
// one FP64 sag evaluation.  Taken only when finite and below 1 cm;
// otherwise the FP64 Newton starts from the conic root as before.
__device__ __forceinline__ void bt_asphere_prestep(const bt_surf& s, const double* pool, double x, double y,
                                                   double vx, double vy, double vz, double* dt) {
    const float fx = (float)(x + vx * *dt), fy = (float)(y + vy * *dt);
    const float r2 = fmaf(fx, fx, fy * fy);
    const ff* c = ff_ptr(pool, s.off + 2 * s.n);
    const ff* dc = c + s.n;
    float pz = 0.f, da = 0.f;
    for (int i = s.n - 1; i >= 0; i--) {
        pz = fmaf(pz, r2, c[i].hi);
        da = fmaf(da, r2, dc[i].hi);
    }
    pz *= r2;
    const float2 cf = *reinterpret_cast<const float2*>(&s.p[11]);  // (1+k)/R^2, 1/R
    const float w = fmaf(-r2, cf.x, 1.0f);
    if (!(w > 0.0f)) return;
    const float kf = fmaf(rsqrtf(w), cf.y, da);  // -(d sag / dr) / r
    const float den = fmaf(-fx * kf, (float)vx, fmaf(-fy * kf, (float)vy, (float)vz));
    const float ddt = pz / den;
    if (fabsf(ddt) < 1e-2f) *dt += (double)ddt;  // false for NaN / inf
}

// Time to intersect for the trace kernels.  PRESTEP: FP32 Newton pre-step
// on aspheres (the batched kernel; same-call A/B: batched +4 %, the plain
// trace -1 %, so the plain trace is built without it).
template <bool PRESTEP = false>
__device__ __forceinline__ bool bt_leaf_tti_fast(const Prog& P, int si, double x, double y, double z, double vx,
                                                 double vy, double vz, double& dt, int niter) {
    const bt_surf& s = P.surfs[si];
    switch (s.kind) {
    case BT_S_SPHERE: {
        const double R = s.p[0];
        const double z0 = z - R;
        const double a = vz * vz + (vx * vx + vy * vy);
        const double b = 2 * vz * z0 + 2 * (vx * x + vy * y);
        const double c = z0 * z0 - s.p[1] + (x * x + y * y);
        // the reference takes max(dt1, dt2) when vz*R < 0, else min; the
        // larger root is the "+sqrt" one when a > 0
        const bool want_max = (vz * R < 0);
        return bt_one_root(a, b, c, want_max == (a > 0), &dt);
    }
    case BT_S_PARABOLOID: {
        const double a = (vx * vx + vy * vy) * s.p[2];
        const double b = (x * vx + y * vy) * s.p[1] - vz;
        const double c = (x * x + y * y) * s.p[2] - z;
        if (a == 0) { dt = -c / b; return true; }
        const bool want_max = (vz * s.p[0] < 0);
        return bt_one_root(a, b, c, want_max == (a > 0), &dt);
    }
    case BT_S_QUADRIC:
    case BT_S_ASPHERE: {
        // conic start (src/quadric.cpp:41-71): root with the smaller |z|
        const double z0 = z - s.p[6];
        const double vrr0 = vx * x + vy * y;
        const double a = vz * vz + (vx * vx + vy * vy) * s.p[5];
        const double b = 2 * (vz * z0 + vrr0 * s.p[5]);
        const double c = z0 * z0 - s.p[7] + (x * x + y * y) * s.p[5];
        double t1, t2;
        if (!bt_quad_roots(a, b, c, &t1, &t2)) return false;
        dt = (fabs(z + vz * t1) < fabs(z + vz * t2)) ? t1 : t2;
        if (s.kind == BT_S_QUADRIC) return true;
        if (PRESTEP && s.n > 0) bt_asphere_prestep(s, P.pool, x, y, vx, vy, vz, &dt);
        return bt_newton_mixed(P, si, x, y, z, vx, vy, vz, dt, niter);
    }
    case BT_S_POLY:
    case BT_S_BICUBIC:
    case BT_S_MODAL:
        return bt_newton_mixed(P, si, x, y, z, vx, vy, vz, dt, niter);
    default: {
        double ux, uy;
        bool slope_ok;
        return bt_leaf_tti(P, si, x, y, z, vx, vy, vz, dt, niter, &ux, &uy, &slope_ok);
    }
    }
}

template <bool PRESTEP = false>
__device__ __forceinline__ bool bt_surf_tti_fast(const Prog& P, int si, double x, double y, double z, double vx,
                                                 double vy, double vz, double& dt, int niter) {
    const bt_surf& s = P.surfs[si];
    if (s.kind != BT_S_SUM) return bt_leaf_tti_fast<PRESTEP>(P, si, x, y, z, vx, vy, vz, dt, niter);
    if (!bt_leaf_tti_fast<PRESTEP>(P, s.m, x, y, z, vx, vy, vz, dt, niter)) return false;
    return bt_newton_mixed(P, si, x, y, z, vx, vy, vz, dt, niter);
}
