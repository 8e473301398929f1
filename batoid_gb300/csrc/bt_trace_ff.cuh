// Float-float path of the fused trace.
//
// The fused trace is bound by the FP64 pipe: on GB300 each FP64-pipe
// instruction (DFMA, DADD, DMUL, compares, double<->float conversions)
// occupies the pipe for the same time, and a stage of the FP64 form costs
// 60-450 of them per ray.  The FP32 pipe issues ~64 lanes for each FP64
// lane.  This path evaluates each stage's geometry in float-float (pairs of
// floats, ~48 significant bits) on float-float copies of the ray, converted
// with integer instructions, and keeps FP64 where the result's stability
// needs it:
//  * the ray's state: positions and directions stay FP64 between stages;
//    the position update x + v dt is an FP64 FMA, so a ray whose direction
//    component is zero keeps that coordinate exactly, as in the reference;
//  * the Newton intersection solve of aspheres, polynomial surfaces and
//    sums: iterated in float-float to ~1e-13 m, then its residual
//    sag(x + v dt) - (z + vz dt) is evaluated in FP64 at the FP64 point and
//    the last correction applied in FP64 (src/surface.cpp:22-49: success is
//    |residual| < 1e-12 at the final point);
//  * the optical path: t accumulates in FP64.
// Analytic intersections (plane, sphere, paraboloid, quadric; quadrics and
// large spheres then corrected by one FP64 Newton step), normals,
// reflection, refraction, the media and the annulus / circle obscuration
// tests run in float-float; an obscuration test within 1e-13 relative of
// its edge falls back to the reference's FP64 test on the FP64 position.
// Results agree with the reference within its parity tolerances
// (positions 1e-12 m, path 1e-11 m).
//
// Stages whose surface kind has no float-float form here (Tilted, Bicubic,
// a Sum over those) and obscurations other than circles and annuli run the
// FP64 form.  The batched kernel's bending-mode tables (a Sum's later
// child) are evaluated in FP32 on their cached corner values.
#pragma once
#include "bt_trace_core.cuh"

// Index of the medium whose index is cached and the cached (n, 1/n).
struct MediumCacheF {
    int idx;
    ff n, inv_n;
};

// Float-float copies of a ray's x, y and direction from the stage that
// produced them (valid while ok): the next stage reuses those its transform
// leaves unchanged instead of converting the FP64 values again.
struct RayCacheF {
    bool ok;
    ff x, y, vx, vy, vz;
};

// |a| < c for finite c > 0 on the integer pipe (false for NaN, as the
// floating-point comparison).
__device__ __forceinline__ bool d_abs_lt(double a, double c) {
    const unsigned long long ua = (unsigned long long)__double_as_longlong(a) & 0x7fffffffffffffffull;
    return ua < (unsigned long long)__double_as_longlong(c);
}

__device__ __forceinline__ ff ff_one() { return ff{1.f, 0.f}; }

// a != 0 (either sign of zero) on the integer pipe.
__device__ __forceinline__ bool d_nonzero(double a) {
    return ((unsigned long long)__double_as_longlong(a) << 1) != 0ull;
}

// ---------------------------------------------------------------------------
// Which surfaces have a float-float form
// ---------------------------------------------------------------------------

__device__ __forceinline__ bool ffs_leaf_ok(const bt_surf& s) {
    switch (s.kind) {
    case BT_S_PLANE:
        return true;
    case BT_S_SPHERE:
    case BT_S_PARABOLOID:
    case BT_S_QUADRIC:
    case BT_S_ASPHERE:
        return s.ffc >= 0 && d_nonzero(s.p[0]);
    case BT_S_POLY:
        return s.ffc >= 0;
    default:
        return false;
    }
}

__device__ __forceinline__ bool ffs_ok(const Prog& P, int si) {
    const bt_surf& s = P.surfs[si];
    if (s.kind != BT_S_SUM) return ffs_leaf_ok(s);
    for (int c = 0; c < s.n; c++) {
        const bt_surf& cs = P.surfs[s.m + c];
        // modal bending tables of the batched kernel (a Sum's later child)
        if (cs.kind == BT_S_MODAL) {
            if (c == 0 || P.mc == nullptr) return false;
        } else if (!ffs_leaf_ok(cs)) {
            return false;
        }
    }
    return true;
}

// MODAL surface (sum of bending-mode tables, batched kernel only): the cell
// and fractions from the float-float position, the per-thread cached corner
// values of the weighted tables (FP32 copies) and the Hermite patch in
// FP32.  The bending sags are ~1e-7 m, so FP32 carries them to ~1e-14 m.
// Returns the sag as *zp, the FP32 slope (-dz/dx, -dz/dy).  Outside the grid
// the reference's fill value (NaN or 0, src/bicubic.cpp:19-40).
static __device__ __noinline__ void ff_modal_eval(const Prog& P, const bt_surf& s, ff x, ff y, ff* zp, float* ux, float* uy) {
    const ff u = ff_mul(ff_sub(x, d_to_ff(s.p[0])), d_to_ff(s.p[6]));
    const ff v = ff_mul(ff_sub(y, d_to_ff(s.p[1])), d_to_ff(s.p[7]));
    float fu = floorf(u.hi), fv = floorf(v.hi);
    if (u.hi == fu && u.lo < 0.f) fu -= 1.f;
    if (v.hi == fv && v.lo < 0.f) fv -= 1.f;
    if (!(fu >= 0.f) || !(fv >= 0.f) || fu >= (float)(s.n - 1) || fv >= (float)(s.m - 1)) {
        const float fill = d_nonzero(s.p[4]) ? __int_as_float(0x7fc00000) : 0.f;
        *zp = ff{fill, 0.f};
        *ux = fill;
        *uy = fill;
        return;
    }
    const int ix = (int)fu, iy = (int)fv;
    const float xf = (u.hi - fu) + u.lo, yf = (v.hi - fv) + v.lo;
    const int cell = iy * s.n + ix;
    int* cellp = P.mcell + threadIdx.x;
    if (*cellp != cell) {
        bt_modal_fill(P.pool, &s, ix, iy, P.mc + threadIdx.x, P.mcf + threadIdx.x, P.mstride);
        *cellp = cell;
    }
    float w[16];
#pragma unroll
    for (int k = 0; k < 16; k++) w[k] = P.mcf[k * P.mstride + threadIdx.x];
    float val, gx, gy;
    bt_hermite<float>(xf, yf, d_to_ff(s.p[2]).hi, d_to_ff(s.p[3]).hi, w, w + 4, w + 8, w + 12, &val, &gx, &gy, true,
                      true);
    *zp = ff{val, 0.f};
    *ux = -gx;
    *uy = -gy;
}

// ---------------------------------------------------------------------------
// Sags (float-float value as conic part + polynomial part, FP32 slope)
// ---------------------------------------------------------------------------

// r^2 = x^2 + y^2
__device__ __forceinline__ ff ff_r2(ff x, ff y) { return ff_add(ff_sqr(x), ff_sqr(y)); }

// Conic sag of a QUADRIC / ASPHERE record, r^2 / (R (1 + q)) with
// q = sqrt(1 - r^2 (1+k)/R^2).  (The equal form (1 - q) R/(1+k), which the
// FP64 form may use, multiplies the rounding of q by |R/(1+k)|, ~100 m for
// some mirrors: in float-float that would be ~1e-12 m.)
__device__ __forceinline__ ff ffs_conic(const double* C, ff r2, ff* w_out) {
    const ff w = ff_sub(ff_one(), ff_mul(r2, ff_slot(C + 4)));
    *w_out = w;
    return ff_div(r2, ff_mul(ff_slot(C + 0), ff_add(ff_one(), ff_sqrt(w))));
}

// Leaf sag at (x, y): *zc the conic part (recomputed in FP64 by
// ffs_conic64), *zp the polynomial part, (ux, uy) the FP32 slope
// (-dz/dx, -dz/dy) for the Newton derivative.
struct SagF {
    ff zc, zp;
    float ux, uy;  // slope (-dz/dx, -dz/dy) of the whole sag, FP32
    float px, py;  // the same for the polynomial part zp alone
};

static __device__ __noinline__ SagF ffs_leaf_eval_o(const bt_surf& s, const double* pool, ff x, ff y) {
    SagF o;
    ff* zc = &o.zc;
    ff* zp = &o.zp;
    float* ux = &o.ux;
    float* uy = &o.uy;
    const double* C = pool + s.ffc;
    *zp = ff{0.f, 0.f};
    o.px = 0.f;
    o.py = 0.f;
    switch (s.kind) {
    case BT_S_SPHERE: {
        // R (1 - q) = r^2 / (R (1 + q)), q = sqrt(1 - r^2/R^2), in the form
        // without cancellation
        const ff r2 = ff_r2(x, y);
        const ff w = ff_sub(ff_one(), ff_mul(r2, ff_slot(C + 3)));
        *zc = ff_div(r2, ff_mul(ff_slot(C + 0), ff_add(ff_one(), ff_sqrt(w))));
        const float k = rsqrtf(w.hi) * ff_slot(C + 2).hi;
        *ux = -x.hi * k;
        *uy = -y.hi * k;
        return o;
    }
    case BT_S_PARABOLOID: {
        *zc = ff_mul(ff_r2(x, y), ff_slot(C + 2));
        const float k = ff_slot(C + 1).hi;
        *ux = -x.hi * k;
        *uy = -y.hi * k;
        return o;
    }
    case BT_S_QUADRIC:
    case BT_S_ASPHERE: {
        const ff r2 = ff_r2(x, y);
        ff w;
        *zc = ffs_conic(C, r2, &w);
        float kf = rsqrtf(w.hi) * ff_slot(C + 5).hi;
        if (s.kind == BT_S_ASPHERE && s.n > 0) {
            const ff* c = ff_ptr(pool, s.off + 2 * s.n);
            const ff* dc = c + s.n;
            *zp = ff_mul(ff_horner(r2, c, s.n), r2);
            float da = 0.f;
            for (int i = s.n - 1; i >= 0; i--) da = fmaf(da, r2.hi, dc[i].hi);
            kf += da;
            o.px = -x.hi * da;
            o.py = -y.hi * da;
        }
        *ux = -x.hi * kf;
        *uy = -y.hi * kf;
        return o;
    }
    case BT_S_POLY: {
        const ff xx = ff_sub(x, ff_slot(C + 0)), yy = ff_sub(y, ff_slot(C + 1));
        const int nx = s.n, ny = s.m;
        const int g = (nx - 1) * (ny - 1);
        const ff* c = ff_ptr(pool, s.off + nx * ny + 2 * g);
        *zc = ff{0.f, 0.f};
        if (d_nonzero(s.p[2])) {  // triangular arrays (Zernike sums)
            *zp = ff_horner2d_tri(xx, yy, c, nx);
            *ux = -f_horner2d_tri(xx.hi, yy.hi, c + nx * ny, nx - 1);
            *uy = -f_horner2d_tri(xx.hi, yy.hi, c + nx * ny + g, nx - 1);
        } else {
            *zp = ff_horner2d(xx, yy, c, nx, ny);
            *ux = -f_horner2d(xx.hi, yy.hi, c + nx * ny, nx - 1, ny - 1);
            *uy = -f_horner2d(xx.hi, yy.hi, c + nx * ny + g, nx - 1, ny - 1);
        }
        o.px = *ux;
        o.py = *uy;
        return o;
    }
    default:  // plane
        *zc = ff{0.f, 0.f};
        *ux = 0.f;
        *uy = 0.f;
        return o;
    }
}

// Out of line (one copy of the code for every caller): the fully inlined
// float-float form missed in the instruction cache on most issues.
__device__ __forceinline__ void ffs_leaf_eval(const bt_surf& s, const double* pool, ff x, ff y, ff* zc, ff* zp,
                                              float* ux, float* uy, float* px = nullptr, float* py = nullptr) {
    const SagF o = ffs_leaf_eval_o(s, pool, x, y);
    *zc = o.zc;
    *zp = o.zp;
    *ux = o.ux;
    *uy = o.uy;
    if (px) {
        *px = o.px;
        *py = o.py;
    }
}

// (px, py), when given: the FP32 slope of the polynomial part alone.
__device__ __forceinline__ void ffs_eval(const Prog& P, int si, ff x, ff y, ff* zc, ff* zp, float* ux, float* uy,
                                         float* px = nullptr, float* py = nullptr) {
    const bt_surf& s = P.surfs[si];
    if (s.kind != BT_S_SUM) {
        ffs_leaf_eval(s, P.pool, x, y, zc, zp, ux, uy, px, py);
        return;
    }
    ff c_acc{0.f, 0.f}, p_acc{0.f, 0.f};
    float gx = 0.f, gy = 0.f, hx = 0.f, hy = 0.f;
    for (int c = 0; c < s.n; c++) {
        ff cz{0.f, 0.f}, pz;
        float cx, cy, qx, qy;
        const bt_surf& cs = P.surfs[s.m + c];
        if (cs.kind == BT_S_MODAL) {
            ff_modal_eval(P, cs, x, y, &pz, &cx, &cy);
            qx = cx;
            qy = cy;
        } else {
            ffs_leaf_eval(cs, P.pool, x, y, &cz, &pz, &cx, &cy, &qx, &qy);
        }
        c_acc = ff_add(c_acc, cz);
        p_acc = ff_add(p_acc, pz);
        gx += cx;
        gy += cy;
        hx += qx;
        hy += qy;
    }
    *zc = c_acc;
    *zp = p_acc;
    *ux = gx;
    *uy = gy;
    if (px) {
        *px = hx;
        *py = hy;
    }
}

// FP64 conic part of the sag (the reference's expressions, src/sphere.cpp,
// src/paraboloid.cpp, src/quadric.cpp) at an FP64 point.
__device__ __forceinline__ double ffs_conic64_leaf(const bt_surf& s, double x, double y) {
    double z, k;
    switch (s.kind) {
    case BT_S_SPHERE:
        bt_sphere_conic(s, x * x + y * y, &z, &k);
        return z;
    case BT_S_PARABOLOID:
        return (x * x + y * y) * s.p[2];
    case BT_S_QUADRIC:
    case BT_S_ASPHERE:
        bt_conic(s, x * x + y * y, &z, &k);
        return z;
    default:
        return 0.0;
    }
}

__device__ __forceinline__ double ffs_conic64(const Prog& P, int si, double x, double y) {
    const bt_surf& s = P.surfs[si];
    if (s.kind != BT_S_SUM) return ffs_conic64_leaf(s, x, y);
    double z = 0.0;
    for (int c = 0; c < s.n; c++) z += ffs_conic64_leaf(P.surfs[s.m + c], x, y);
    return z;
}

// ---------------------------------------------------------------------------
// Intersections
// ---------------------------------------------------------------------------

// One root of a t^2 + b t + c = 0 as bt_one_root (the reference's dt1 / dt2
// pair, src/sphere.cpp:51-58): `plus` selects (-b + sqrt(D)) / 2a.
__device__ __forceinline__ bool ff_one_root(ff a, ff b, ff c, bool plus, ff* t) {
    const ff disc = ff_sub(ff_sqr(b), ff_mul_f(ff_mul(a, c), 4.f));
    if (disc.hi < 0.f) return false;
    const ff s = ff_sqrt(disc);
    const ff mb = ff_neg(b);
    if (b.hi > 0.f) *t = plus ? ff_div(ff_mul_f(c, 2.f), ff_sub(mb, s)) : ff_div(ff_sub(mb, s), ff_mul_f(a, 2.f));
    else *t = plus ? ff_div(ff_add(mb, s), ff_mul_f(a, 2.f)) : ff_div(ff_mul_f(c, 2.f), ff_add(mb, s));
    return true;
}

// Conic root with the smaller |z| (src/quadric.cpp:41-71).
struct RootF {
    ff dt;
    bool ok;
};

__device__ __forceinline__ RootF ff_quadric_root_inl(const double* C, ff x, ff y, ff z, ff vx, ff vy, ff vz) {
    RootF o;
    o.ok = false;
    ff* dt = &o.dt;
    const ff icp1 = ff_slot(C + 1);
    const ff z0 = ff_sub(z, ff_slot(C + 2));
    const ff vrr0 = ff_add(ff_mul(vx, x), ff_mul(vy, y));
    const ff a = ff_add(ff_sqr(vz), ff_mul(ff_r2(vx, vy), icp1));
    const ff b = ff_mul_f(ff_add(ff_mul(vz, z0), ff_mul(vrr0, icp1)), 2.f);
    const ff c = ff_add(ff_sub(ff_sqr(z0), ff_slot(C + 3)), ff_mul(ff_r2(x, y), icp1));
    const ff disc = ff_sub(ff_sqr(b), ff_mul_f(ff_mul(a, c), 4.f));
    if (disc.hi < 0.f) return o;
    const ff s = ff_sqrt(disc);
    const ff mb = ff_neg(b);
    const ff r1 = (b.hi > 0.f) ? ff_div(ff_sub(mb, s), ff_mul_f(a, 2.f)) : ff_div(ff_mul_f(c, 2.f), ff_add(mb, s));
    const ff r2 = ff_div(c, ff_mul(a, r1));
    const ff z1 = ff_mad(vz, r1, z), z2 = ff_mad(vz, r2, z);
    *dt = ff_lt(ff_abs(z1), ff_abs(z2)) ? r1 : r2;
    o.ok = true;
    return o;
}


static __device__ __noinline__ RootF ff_quadric_root_o(const double* C, ff x, ff y, ff z, ff vx, ff vy, ff vz) {
    RootF o;
    o.ok = false;
    ff* dt = &o.dt;
    const ff icp1 = ff_slot(C + 1);
    const ff z0 = ff_sub(z, ff_slot(C + 2));
    const ff vrr0 = ff_add(ff_mul(vx, x), ff_mul(vy, y));
    const ff a = ff_add(ff_sqr(vz), ff_mul(ff_r2(vx, vy), icp1));
    const ff b = ff_mul_f(ff_add(ff_mul(vz, z0), ff_mul(vrr0, icp1)), 2.f);
    const ff c = ff_add(ff_sub(ff_sqr(z0), ff_slot(C + 3)), ff_mul(ff_r2(x, y), icp1));
    const ff disc = ff_sub(ff_sqr(b), ff_mul_f(ff_mul(a, c), 4.f));
    if (disc.hi < 0.f) return o;
    const ff s = ff_sqrt(disc);
    const ff mb = ff_neg(b);
    const ff r1 = (b.hi > 0.f) ? ff_div(ff_sub(mb, s), ff_mul_f(a, 2.f)) : ff_div(ff_mul_f(c, 2.f), ff_add(mb, s));
    const ff r2 = ff_div(c, ff_mul(a, r1));
    const ff z1 = ff_mad(vz, r1, z), z2 = ff_mad(vz, r2, z);
    *dt = ff_lt(ff_abs(z1), ff_abs(z2)) ? r1 : r2;
    o.ok = true;
    return o;
}

__device__ __forceinline__ bool ff_quadric_root(const double* C, ff x, ff y, ff z, ff vx, ff vy, ff vz, ff* dt) {
    const RootF o = ff_quadric_root_o(C, x, y, z, vx, vy, vz);
    *dt = o.dt;
    return o.ok;
}

// Analytic time to intersect of PLANE / SPHERE / PARABOLOID / QUADRIC.
__device__ __forceinline__ bool ff_analytic_in(const bt_surf& s, const double* pool, ff x, ff y, ff z, ff vx, ff vy,
                                               ff vz, ff* dt) {
    const double* C = pool + s.ffc;
    switch (s.kind) {
    case BT_S_PLANE:
        // src/plane.cpp:23-30
        if (vz.hi == 0.f) return false;
        *dt = ff_div(ff_neg(z), vz);
        return true;
    case BT_S_SPHERE: {
        // src/sphere.cpp:36-67
        const ff R = ff_slot(C + 0);
        const ff z0 = ff_sub(z, R);
        const ff a = ff_add(ff_sqr(vz), ff_r2(vx, vy));
        const ff b = ff_mul_f(ff_add(ff_mul(vz, z0), ff_add(ff_mul(vx, x), ff_mul(vy, y))), 2.f);
        const ff c = ff_add(ff_sub(ff_sqr(z0), ff_slot(C + 1)), ff_r2(x, y));
        const bool want_max = (vz.hi * R.hi < 0.f);
        return ff_one_root(a, b, c, want_max == (a.hi > 0.f), dt);
    }
    case BT_S_PARABOLOID: {
        // src/paraboloid.cpp:38-71
        const ff a = ff_mul(ff_r2(vx, vy), ff_slot(C + 2));
        const ff b = ff_sub(ff_mul(ff_add(ff_mul(x, vx), ff_mul(y, vy)), ff_slot(C + 1)), vz);
        const ff c = ff_sub(ff_mul(ff_r2(x, y), ff_slot(C + 2)), z);
        if (a.hi == 0.f) {
            *dt = ff_div(ff_neg(c), b);
            return true;
        }
        const bool want_max = (vz.hi * ff_slot(C + 0).hi < 0.f);
        return ff_one_root(a, b, c, want_max == (a.hi > 0.f), dt);
    }
    default:  // QUADRIC
        return ff_quadric_root(C, x, y, z, vx, vy, vz, dt);
    }
}

static __device__ __noinline__ RootF ff_analytic_o(const bt_surf& s, const double* pool, ff x, ff y, ff z, ff vx,
                                                   ff vy, ff vz) {
    RootF o;
    o.ok = ff_analytic_in(s, pool, x, y, z, vx, vy, vz, &o.dt);
    return o;
}

// (A plane's root inline: the call would cost more than the root.)
__device__ __forceinline__ bool ff_analytic(const bt_surf& s, const double* pool, ff x, ff y, ff z, ff vx, ff vy,
                                            ff vz, ff* dt) {
    if (s.kind == BT_S_PLANE) {
        if (vz.hi == 0.f) return false;
        *dt = ff_div(ff_neg(z), vz);
        return true;
    }
    const RootF o = ff_analytic_o(s, pool, x, y, z, vx, vy, vz);
    *dt = o.dt;
    return o.ok;
}


// Newton's tangent-plane iteration in float-float from dt, at most niter
// corrections, stopping once a correction is below 1e-7 m: with an FP32
// derivative (relative error ~1e-7) the error left after that correction is
// ~1e-14 m, and the FP64 step that follows (ff_newton_tti) finishes the
// solve.  Returns whether it stopped that way; *zp is the polynomial part
// of the sag carried to the corrected point (first order in the correction,
// FP32 slope: the remainder is ~1e-17 m) and *inv_den 1/F' of the last
// evaluation.
// (Evaluating the polynomial terms in FP32 during the first iterations was
// measured at half the throughput: FP32 rounding of the cancelling terms of
// the Cartesian Zernike arrays keeps the corrections above any useful
// switch-over threshold, so the iterations run out.)
__device__ __forceinline__ bool ff_newton_iter_in(const Prog& P, int si, ff x, ff y, ff z, ff vx, ff vy, ff vz,
                                                  ff* dt, int niter, ff* zp, float* inv_den) {
    const float fvx = vx.hi, fvy = vy.hi, fvz = vz.hi;
    for (int it = 0; it < niter; it++) {
        const ff px = ff_mad(vx, *dt, x), py = ff_mad(vy, *dt, y), pz = ff_mad(vz, *dt, z);
        ff zc;
        float ux, uy, qx, qy;
        ffs_eval(P, si, px, py, &zc, zp, &ux, &uy, &qx, &qy);
        const ff res = ff_sub(ff_add(zc, *zp), pz);
        *inv_den = f_rcp_approx(fmaf(ux, fvx, fmaf(uy, fvy, fvz)));
        const ff ddt = ff_mul_f(res, *inv_den);
        *dt = ff_add(*dt, ddt);
        if (fabsf(ddt.hi) < 1e-7f) {
            // zp at the corrected point: dzp = -(qx vx + qy vy) ddt
            *zp = ff_add_f(*zp, -fmaf(qx, fvx, qy * fvy) * ddt.hi);
            return true;
        }
    }
    return false;
}

struct NewtonF {
    ff dt, zp;
    float inv_den;
    bool conv;
};

static __device__ __noinline__ NewtonF ff_newton_iter_o(const Prog& P, int si, ff x, ff y, ff z, ff vx, ff vy,
                                                       ff vz, ff dt0, int niter) {
    NewtonF o;
    o.dt = dt0;
    o.zp = ff{0.f, 0.f};
    o.inv_den = 0.f;
    o.conv = ff_newton_iter_in(P, si, x, y, z, vx, vy, vz, &o.dt, niter, &o.zp, &o.inv_den);
    return o;
}

__device__ __forceinline__ bool ff_newton_iter(const Prog& P, int si, ff x, ff y, ff z, ff vx, ff vy, ff vz, ff* dt,
                                               int niter, ff* zp, float* inv_den) {
    const NewtonF o = ff_newton_iter_o(P, si, x, y, z, vx, vy, vz, *dt, niter);
    *dt = o.dt;
    *zp = o.zp;
    *inv_den = o.inv_den;
    return o.conv;
}


// Residual of surface si at dt in float-float (for a first child's success
// test, as the reference's |sag - z| < 1e-12 at its final point).
__device__ __forceinline__ bool ff_residual_ok(const Prog& P, int si, ff x, ff y, ff z, ff vx, ff vy, ff vz, ff dt) {
    const ff px = ff_mad(vx, dt, x), py = ff_mad(vy, dt, y), pz = ff_mad(vz, dt, z);
    ff zc, zp;
    float ux, uy;
    ffs_eval(P, si, px, py, &zc, &zp, &ux, &uy);
    const ff res = ff_sub(ff_add(zc, zp), pz);
    return fabsf(res.hi) < 1e-12f;
}

// FP64 state of a ray in a surface's frame, with its float-float copy.
// Passed by value to the out-of-line helpers (in registers); by reference
// it had to live on each thread's stack.
struct RayLocal {
    double xd, yd, zd, vxd, vyd, vzd;
    ff x, y, z, vx, vy, vz;
};

// Iterative intersection of an ASPHERE / POLY / SUM: start t0 (the conic
// root, 0, or the first child's own solve: src/asphere.cpp:76-85,
// src/sum.cpp:47-56), float-float Newton, then the FP64 residual at the FP64
// point and the final correction in FP64.  On success *dt_out is the FP64 dt.
//
// The float-float iterations run on the ray re-anchored at its FP64 point
// p0 = x + v t0 (FP64 FMAs), in the offset d = dt - t0: the residual's terms
// are then of the size of the sag, not of the distance the ray travelled
// (15 m before the primary of a telescope), so their rounding (~1e-16 m)
// Inside the out-of-line Newton solve, the starting quadric root and the
// Newton loop are inline where BT_FF_INLINE_NEWTON is 1 (the plain trace:
// measured 4 % faster) and calls elsewhere (the batched kernel, whose
// Sums with a bending-mode child measured 15 % slower inline).
#ifndef BT_FF_INLINE_NEWTON
#define BT_FF_INLINE_NEWTON 0
#endif
#ifndef BT_FF_INLINE_QROOT
#define BT_FF_INLINE_QROOT BT_FF_INLINE_NEWTON
#endif
#ifndef BT_FF_INLINE_NORMAL
#define BT_FF_INLINE_NORMAL BT_FF_INLINE_NEWTON
#endif
#if BT_FF_INLINE_QROOT
#define BT_FF_QROOT ff_quadric_root_inl
#else
#define BT_FF_QROOT ff_quadric_root_o
#endif
#if BT_FF_INLINE_NEWTON
#define BT_FF_NEWTON ff_newton_iter_in
#else
#define BT_FF_NEWTON ff_newton_iter
#endif

// stays far below the 1e-12 m convergence and success thresholds.
static __device__ __noinline__ bool ff_newton_tti(const Prog& P, int si, const RayLocal L, int niter, double* dt_out) {
    const bt_surf& s = P.surfs[si];
    const ff vx = L.vx, vy = L.vy, vz = L.vz;
    ff t0{0.f, 0.f};
    bool child_done = false;
    int c0 = -1;
    if (s.kind == BT_S_SUM) {
        c0 = s.m;
        const bt_surf& first = P.surfs[c0];
        if (first.kind == BT_S_ASPHERE) {
            {
                const RootF q = BT_FF_QROOT(P.pool + first.ffc, L.x, L.y, L.z, vx, vy, vz);
                if (!q.ok) return false;
                t0 = q.dt;
            }
        } else if (first.kind != BT_S_POLY) {
            if (!ff_analytic(first, P.pool, L.x, L.y, L.z, vx, vy, vz, &t0)) return false;
            child_done = true;
        }
    } else if (s.kind == BT_S_ASPHERE) {
        {
            const RootF q = BT_FF_QROOT(P.pool + s.ffc, L.x, L.y, L.z, vx, vy, vz);
            if (!q.ok) return false;
            t0 = q.dt;
        }
    }
    // anchor
    const double t0d = ff_to_d(t0);
    const double p0x = fma(L.vxd, t0d, L.xd), p0y = fma(L.vyd, t0d, L.yd), p0z = fma(L.vzd, t0d, L.zd);
    const ff ax = d_to_ff(p0x), ay = d_to_ff(p0y), az = d_to_ff(p0z);
    ff d{0.f, 0.f};
    ff zp;
    float inv_den = 0.f;
    if (c0 >= 0 && !child_done) {
        // the first child's own Newton; it must succeed (src/sum.cpp:47-56)
        if (!BT_FF_NEWTON(P, c0, ax, ay, az, vx, vy, vz, &d, niter, &zp, &inv_den) &&
            !ff_residual_ok(P, c0, ax, ay, az, vx, vy, vz, d))
            return false;
    }
    const bool conv = BT_FF_NEWTON(P, si, ax, ay, az, vx, vy, vz, &d, niter, &zp, &inv_den);
    // FP64 residual at the FP64 point x + v dt
    double dtd = t0d + ff_to_d(d);
    const double px = fma(L.vxd, dtd, L.xd), py = fma(L.vyd, dtd, L.yd), pz = fma(L.vzd, dtd, L.zd);
    if (!conv) {
        // no correction below 1e-12 within niter: the polynomial part at
        // this dt for the final test below
        ff zc;
        float ux, uy;
        ffs_eval(P, si, ff_mad(vx, d, ax), ff_mad(vy, d, ay), &zc, &zp, &ux, &uy);
    }
    // (after a converged iteration zp was carried to this point)
    double res = ffs_conic64(P, si, px, py) + ff_to_d(zp) - pz;
    bool ok = d_abs_lt(res, 1e-12);
    // converged: the residual after this last correction is ~1e-7 of |res|;
    // otherwise, as the reference after its niter iterations, success is
    // |residual| < 1e-12 at the final point
    if (conv && ok) dtd += res * f2d_bits(inv_den);
    if (conv && !ok) {
        // converged in float-float but not yet to 1e-12 in FP64 (should not
        // happen; kept as a safety net): up to two FP64 corrections, the
        // polynomial part re-evaluated at each point
        for (int k = 0; k < 2 && !ok; k++) {
            dtd += res * f2d_bits(inv_den);
            const double qx = fma(L.vxd, dtd, L.xd), qy = fma(L.vyd, dtd, L.yd), qz = fma(L.vzd, dtd, L.zd);
            ff zc;
            float ux, uy;
            ffs_eval(P, si, d_to_ff(qx), d_to_ff(qy), &zc, &zp, &ux, &uy);
            res = ffs_conic64(P, si, qx, qy) + ff_to_d(zp) - qz;
            ok = d_abs_lt(res, 1e-12);
        }
    }
    *dt_out = dtd;
    return ok;
}

// Analytic roots whose float-float rounding can approach the position
// tolerance (|R| above 50 m for spheres and paraboloids, every quadric: the
// quadric form subtracts squares of R/(1+k), thousands of metres for
// near-parabolic mirrors) are corrected by one FP64 Newton step on the
// surface's FP64 sag.  Success stays the analytic root's (a finite
// discriminant), as in the reference; the step is applied only when the
// residual is finite and below 1e-9 m.
static __device__ __noinline__ double ff_refine64(const Prog& P, int si, const RayLocal L, ff dt) {
    double dtd = ff_to_d(dt);
    const double px = fma(L.vxd, dtd, L.xd), py = fma(L.vyd, dtd, L.yd), pz = fma(L.vzd, dtd, L.zd);
    ff zc, zp;
    float ux, uy;
    ffs_eval(P, si, ff_mad(L.vx, dt, L.x), ff_mad(L.vy, dt, L.y), &zc, &zp, &ux, &uy);
    const double res = ffs_conic64(P, si, px, py) - pz;
    if (d_abs_lt(res, 1e-9)) dtd += res * f2d_bits(f_rcp_approx(fmaf(ux, L.vx.hi, fmaf(uy, L.vy.hi, L.vz.hi))));
    return dtd;
}

__device__ __forceinline__ bool ffs_needs_refine(const bt_surf& s) {
    if (s.kind == BT_S_QUADRIC) return true;
    if (s.kind == BT_S_SPHERE || s.kind == BT_S_PARABOLOID) return !d_abs_lt(s.p[0], 50.0);
    return false;
}

// ---------------------------------------------------------------------------
// Normals, reflection, refraction
// ---------------------------------------------------------------------------

// Slope (ux, uy) = (nx/nz, ny/nz) of a leaf at (x, y), float-float.
struct SlopeF {
    ff ux, uy;
};

static __device__ __noinline__ SlopeF ffs_leaf_slope_o(const bt_surf& s, const double* pool, ff x, ff y) {
    SlopeF o;
    ff* ux = &o.ux;
    ff* uy = &o.uy;
    const double* C = pool + s.ffc;
    switch (s.kind) {
    case BT_S_SPHERE: {
        const ff w = ff_sub(ff_one(), ff_mul(ff_r2(x, y), ff_slot(C + 3)));
        const ff k = ff_mul(ff_slot(C + 2), ff_rsqrt(w));
        *ux = ff_neg(ff_mul(x, k));
        *uy = ff_neg(ff_mul(y, k));
        return o;
    }
    case BT_S_PARABOLOID: {
        const ff k = ff_slot(C + 1);
        *ux = ff_neg(ff_mul(x, k));
        *uy = ff_neg(ff_mul(y, k));
        return o;
    }
    case BT_S_QUADRIC:
    case BT_S_ASPHERE: {
        const ff r2 = ff_r2(x, y);
        const ff w = ff_sub(ff_one(), ff_mul(r2, ff_slot(C + 4)));
        ff k = ff_mul(ff_slot(C + 5), ff_rsqrt(w));
        if (s.kind == BT_S_ASPHERE && s.n > 0) k = ff_add(k, ff_horner(r2, ff_ptr(pool, s.off + 3 * s.n), s.n));
        *ux = ff_neg(ff_mul(x, k));
        *uy = ff_neg(ff_mul(y, k));
        return o;
    }
    case BT_S_POLY: {
        const int nx = s.n, ny = s.m;
        const int g = (nx - 1) * (ny - 1);
        const ff* c = ff_ptr(pool, s.off + nx * ny + 2 * g);
        const ff xx = ff_sub(x, ff_slot(C + 0)), yy = ff_sub(y, ff_slot(C + 1));
        if (d_nonzero(s.p[2])) {
            *ux = ff_neg(ff_horner2d_tri(xx, yy, c + nx * ny, nx - 1));
            *uy = ff_neg(ff_horner2d_tri(xx, yy, c + nx * ny + g, nx - 1));
        } else {
            *ux = ff_neg(ff_horner2d(xx, yy, c + nx * ny, nx - 1, ny - 1));
            *uy = ff_neg(ff_horner2d(xx, yy, c + nx * ny + g, nx - 1, ny - 1));
        }
        return o;
    }
    default:
        *ux = ff{0.f, 0.f};
        *uy = ff{0.f, 0.f};
        return o;
    }
}

__device__ __forceinline__ void ffs_leaf_slope(const bt_surf& s, const double* pool, ff x, ff y, ff* ux, ff* uy) {
    const SlopeF o = ffs_leaf_slope_o(s, pool, x, y);
    *ux = o.ux;
    *uy = o.uy;
}

// Unit normal at (x, y) with the reference's conventions (bt_normal_precise).
struct Vec3F {
    ff x, y, z;
};

__device__ __forceinline__ void ffs_normal_in(const Prog& P, int si, ff x, ff y, ff* nx, ff* ny, ff* nz);

static __device__ __noinline__ Vec3F ffs_normal_o(const Prog& P, int si, ff x, ff y) {
    Vec3F o;
    ffs_normal_in(P, si, x, y, &o.x, &o.y, &o.z);
    return o;
}

// (Plane and sphere normals inline: a few float-float operations, cheaper
// than the call.)
__device__ __forceinline__ void ffs_normal(const Prog& P, int si, ff x, ff y, ff* nx, ff* ny, ff* nz) {
#if BT_FF_INLINE_NORMAL
    ffs_normal_in(P, si, x, y, nx, ny, nz);
    return;
#endif
    const bt_surf& s = P.surfs[si];
    if (s.kind == BT_S_PLANE || s.kind == BT_S_SPHERE) {
        ffs_normal_in(P, si, x, y, nx, ny, nz);
        return;
    }
    const Vec3F o = ffs_normal_o(P, si, x, y);
    *nx = o.x;
    *ny = o.y;
    *nz = o.z;
}

__device__ __forceinline__ void ffs_normal_in(const Prog& P, int si, ff x, ff y, ff* nx, ff* ny, ff* nz) {
    const bt_surf& s = P.surfs[si];
    if (s.kind == BT_S_PLANE) {
        *nx = ff{0.f, 0.f}; *ny = ff{0.f, 0.f}; *nz = ff_one();
        return;
    }
    if (s.kind == BT_S_SPHERE) {
        // (-x/R, -y/R, sqrt(1 - r^2/R^2))
        const double* C = P.pool + s.ffc;
        const ff iR = ff_slot(C + 2);
        *nx = ff_neg(ff_mul(x, iR));
        *ny = ff_neg(ff_mul(y, iR));
        *nz = ff_sqrt(ff_sub(ff_one(), ff_mul(ff_r2(x, y), ff_slot(C + 3))));
        return;
    }
    ff ux{0.f, 0.f}, uy{0.f, 0.f};
    if (s.kind != BT_S_SUM) {
        ffs_leaf_slope(s, P.pool, x, y, &ux, &uy);
    } else {
        for (int c = 0; c < s.n; c++) {
            ff cx, cy;
            const bt_surf& cs = P.surfs[s.m + c];
            if (cs.kind == BT_S_MODAL) {
                ff z;
                float gx, gy;
                ff_modal_eval(P, cs, x, y, &z, &gx, &gy);
                cx = ff{gx, 0.f};
                cy = ff{gy, 0.f};
            } else {
                ffs_leaf_slope(cs, P.pool, x, y, &cx, &cy);
            }
            ux = ff_add(ux, cx);
            uy = ff_add(uy, cy);
        }
    }
    const ff k = ff_rsqrt(ff_add_f(ff_r2(ux, uy), 1.f));
    *nx = ff_mul(ux, k);
    *ny = ff_mul(uy, k);
    *nz = k;
}

__device__ __forceinline__ ff ff_dot3(ff ax, ff ay, ff az, ff bx, ff by, ff bz) {
    return ff_add(ff_add(ff_mul(ax, bx), ff_mul(ay, by)), ff_mul(az, bz));
}

// Refractive index and its reciprocal in float-float (src/medium.cpp).
static __device__ __noinline__ void ff_medium(const Prog& P, int mi, double w, ff* n, ff* inv_n) {
    const bt_medium& m = P.media[mi];
    if (m.kind == BT_M_CONST) {
        *n = ff_slot(&m.p[2]);
        *inv_n = ff_slot(&m.p[3]);
        return;
    }
    if (m.kind == BT_M_SELLMEIER) {
        // src/medium.cpp:145-149: n^2 = 1 + sum B_i x / (x - C_i), x = (w / 1 um)^2
        const ff wf = d_to_ff(w);
        // 1e12 = 999999995904 + 4096, both exact floats
        const ff x = ff_mul(ff_sqr(wf), ff{999999995904.f, 4096.f});
        const double* C = P.pool + m.off;  // B1..B3, C1..C3 as float-float pairs
        ff n2 = ff_one();
        for (int i = 0; i < 3; i++) n2 = ff_add(n2, ff_div(ff_mul(ff_slot(C + i), x), ff_sub(x, ff_slot(C + 3 + i))));
        *n = ff_sqrt(n2);
        *inv_n = ff_div(ff_one(), *n);
        return;
    }
    const double nd = bt_getN(P, mi, w);
    *n = d_to_ff(nd);
    *inv_n = d_to_ff(1.0 / nd);
}

// ---------------------------------------------------------------------------
// Obscurations: circles and annuli in float-float, the rest in FP64
// ---------------------------------------------------------------------------

// hypot(dx, dy) < r decided from h^2 - r^2 in float-float unless within
// 1e-13 relative of r^2; then *undecided.  rf: r as a float-float pair.
__device__ __forceinline__ bool ff_radius_less(ff dx, ff dy, ff rf, double r, bool* undecided) {
    // clear cases in FP32 first (h^2 and r^2 to ~3e-7 relative)
    const float h2f = fmaf(dx.hi, dx.hi, dy.hi * dy.hi), r2f = rf.hi * rf.hi;
    if (h2f < r2f * (1.f - 1e-5f)) return __double_as_longlong(r) > 0;
    if (h2f > r2f * (1.f + 1e-5f)) return false;
    const ff r2 = ff_sqr(rf);
    const ff d = ff_sub(ff_r2(dx, dy), r2);
    const float thr = 1e-13f * r2.hi;
    if (d.hi < -thr) return __double_as_longlong(r) > 0;  // r > 0 (a finite radius)
    if (d.hi > thr) return false;
    *undecided = true;
    return false;
}

static __device__ __noinline__ bool ff_obsc_run(const Prog& P, int begin, int end, ff x, ff y, double xd,
                                                double yd) {
    uint32_t stack = 0;
    int sp = 0;
    for (int k = begin; k < end; k++) {
        const bt_obsc& o = P.obsc[k];
        bool v = false;
        if (o.op == BT_O_CIRCLE || o.op == BT_O_ANNULUS) {
            // float-float copies packed by the host: CIRCLE p3..p5 = r, x0,
            // y0; ANNULUS p4, p5 = inner, outer (centre converted if nonzero)
            ff dx = x, dy = y;
            bool und = false;
            if (o.op == BT_O_CIRCLE) {
                dx = ff_sub(x, ff_slot(&o.p[4]));
                dy = ff_sub(y, ff_slot(&o.p[5]));
                v = ff_radius_less(dx, dy, ff_slot(&o.p[3]), o.p[0], &und);
            } else {
                if (d_nonzero(o.p[2])) dx = ff_sub(x, d_to_ff(o.p[2]));
                if (d_nonzero(o.p[3])) dy = ff_sub(y, d_to_ff(o.p[3]));
                const bool in_inner = ff_radius_less(dx, dy, ff_slot(&o.p[4]), o.p[0], &und);
                const bool in_outer = ff_radius_less(dx, dy, ff_slot(&o.p[5]), o.p[1], &und);
                v = !in_inner && in_outer;
            }
            if (und) v = bt_obsc_run(P, k, k + 1, xd, yd);
        } else if (o.op == BT_O_NEGATION || o.op == BT_O_UNION || o.op == BT_O_INTERSECTION) {
            if (o.op == BT_O_NEGATION) {
                sp--;
                v = !((stack >> sp) & 1u);
            } else if (o.op == BT_O_UNION) {
                bool acc = false;
                for (int j = 0; j < o.n; j++) { sp--; acc |= (bool)((stack >> sp) & 1u); }
                v = acc;
            } else {
                bool acc = true;
                for (int j = 0; j < o.n; j++) { sp--; acc &= (bool)((stack >> sp) & 1u); }
                v = acc;
            }
        } else {
            v = bt_obsc_run(P, k, k + 1, xd, yd);
        }
        stack = (stack & ~(1u << sp)) | ((uint32_t)v << sp);
        sp++;
    }
    return sp > 0 ? (bool)((stack >> (sp - 1)) & 1u) : false;
}

// ---------------------------------------------------------------------------
// One stage (semantics of run_stage, src/batoid.cpp:175-506)
// ---------------------------------------------------------------------------

// A stage on the FP64 form, for the surface kinds without a float-float
// form (out of line: rare, and large).
static __device__ __noinline__ void ff_stage_fp64(const Prog& P, const bt_stage& st, RayState& r, int niter) {
    int cm = -1;
    double cn = 0.0, cin = 0.0;
    run_stage<false>(P, st, r, niter, cm, cn, cin);
}

__device__ __forceinline__ void run_stage_ff(const Prog& P, const bt_stage& st, RayState& r, int niter,
                                             MediumCacheF& mc, RayCacheF& fc) {
    if (st.kind == BT_ST_SCREEN || (st.kind != BT_ST_OBSCURE && !r.fail && !ffs_ok(P, st.surf))) {
        ff_stage_fp64(P, st, r, niter);
        fc.ok = false;
        return;
    }
    ff fx, fy;  // float-float copy of the final (x, y), for the obscuration
    bool have_f = false;
    if (st.kind != BT_ST_OBSCURE && !r.fail) {
        RayLocal L;
        // the transform in FP64, as the reference (src/batoid.cpp:225-233)
        if (st.identity == 1) {
            L.xd = r.x; L.yd = r.y; L.zd = r.z; L.vxd = r.vx; L.vyd = r.vy; L.vzd = r.vz;
        } else if (st.identity == 2) {
            L.xd = r.x - st.dr[0]; L.yd = r.y - st.dr[1]; L.zd = r.z - st.dr[2];
            L.vxd = r.vx; L.vyd = r.vy; L.vzd = r.vz;
        } else {
            const double dx = r.x - st.dr[0], dy = r.y - st.dr[1], dz = r.z - st.dr[2];
            L.xd = dx * st.drot[0] + dy * st.drot[3] + dz * st.drot[6];
            L.yd = dx * st.drot[1] + dy * st.drot[4] + dz * st.drot[7];
            L.zd = dx * st.drot[2] + dy * st.drot[5] + dz * st.drot[8];
            L.vxd = r.vx * st.drot[0] + r.vy * st.drot[3] + r.vz * st.drot[6];
            L.vyd = r.vx * st.drot[1] + r.vy * st.drot[4] + r.vz * st.drot[7];
            L.vzd = r.vx * st.drot[2] + r.vy * st.drot[5] + r.vz * st.drot[8];
        }
        // float-float copies; those the transform leaves unchanged come from
        // the previous stage
        const bool same_v = fc.ok && st.identity != 0;
        L.x = (same_v && !d_nonzero(st.dr[0])) ? fc.x : d_to_ff(L.xd);
        L.y = (same_v && !d_nonzero(st.dr[1])) ? fc.y : d_to_ff(L.yd);
        L.z = d_to_ff(L.zd);
        if (same_v) {
            L.vx = fc.vx; L.vy = fc.vy; L.vz = fc.vz;
        } else {
            L.vx = d_to_ff(L.vxd); L.vy = d_to_ff(L.vyd); L.vz = d_to_ff(L.vzd);
        }
        const bt_surf& s = P.surfs[st.surf];
        bool ok;
        double dtd = 0.0;
        if (s.kind == BT_S_ASPHERE || s.kind == BT_S_POLY || s.kind == BT_S_SUM) {
            ok = ff_newton_tti(P, st.surf, L, niter, &dtd);
        } else {
            ff dt;
            ok = ff_analytic(s, P.pool, L.x, L.y, L.z, L.vx, L.vy, L.vz, &dt);
            if (ok) dtd = ffs_needs_refine(s) ? ff_refine64(P, st.surf, L, dt) : ff_to_d(dt);
        }
        if (ok) {
            // src/batoid.cpp:236-242: x += v dt, t += dt
            const double x = fma(L.vxd, dtd, L.xd), y = fma(L.vyd, dtd, L.yd), z = fma(L.vzd, dtd, L.zd);
            double vx = L.vxd, vy = L.vyd, vz = L.vzd;
            r.t += dtd;
            fx = d_to_ff(x);
            fy = d_to_ff(y);
            have_f = true;
            fc.vx = L.vx; fc.vy = L.vy; fc.vz = L.vz;
            if (st.kind == BT_ST_INTERSECT) {
                if (st.coated) r.f *= st.coat_t;
            } else {
                ff nx_, ny_, nz_;
                ffs_normal(P, st.surf, fx, fy, &nx_, &ny_, &nz_);
                const ff wx = L.vx, wy = L.vy, wz = L.vz;
                if (st.kind == BT_ST_REFLECT) {
                    // src/batoid.cpp:343-353
                    const ff a2 = ff_mul_f(ff_dot3(wx, wy, wz, nx_, ny_, nz_), 2.f);
                    fc.vx = ff_sub(wx, ff_mul(a2, nx_));
                    fc.vy = ff_sub(wy, ff_mul(a2, ny_));
                    fc.vz = ff_sub(wz, ff_mul(a2, nz_));
                    vx = ff_to_d(fc.vx);
                    vy = ff_to_d(fc.vy);
                    vz = ff_to_d(fc.vz);
                    if (st.coated) r.f *= st.coat_r;
                } else {
                    // src/batoid.cpp:453-499
                    const ff n1 = ff_rsqrt(ff_add(ff_sqr(wz), ff_r2(wx, wy)));
                    const ff nvx = ff_mul(wx, n1), nvy = ff_mul(wy, n1), nvz = ff_mul(wz, n1);
                    ff alpha = ff_dot3(nvx, nvy, nvz, nx_, ny_, nz_);
                    if (alpha.hi > 0.f) {
                        nx_ = ff_neg(nx_); ny_ = ff_neg(ny_); nz_ = ff_neg(nz_);
                        alpha = ff_neg(alpha);
                    }
                    // 1/n2: a constant medium's from its record; others
                    // cached per ray (a lens's glass between its faces'
                    // vacuum gaps is evaluated once)
                    const int mi = st.medium;
                    const bt_medium& md = P.media[mi];
                    ff inv_n2;
                    if (md.kind == BT_M_CONST) {
                        inv_n2 = ff_slot(&md.p[3]);
                    } else {
                        if (mi != mc.idx) {
                            ff_medium(P, mi, r.w, &mc.n, &mc.inv_n);
                            mc.idx = mi;
                        }
                        inv_n2 = mc.inv_n;
                    }
                    const ff eta = ff_mul(n1, inv_n2);
                    const ff sinsqr = ff_mul(ff_sqr(eta), ff_sub(ff_one(), ff_sqr(alpha)));
                    if (sinsqr.hi > 1.f || (sinsqr.hi == 1.f && sinsqr.lo > 0.f)) {
                        vx = NAN; vy = NAN; vz = NAN;
                        r.fail = true;
                        r.vig = true;
                    } else {
                        // (eta v^ - (eta alpha + cos) n) / n2
                        const ff cosr = ff_sqrt(ff_sub(ff_one(), sinsqr));
                        const ff a = ff_mul(eta, inv_n2);
                        const ff b = ff_mul(ff_add(ff_mul(eta, alpha), cosr), inv_n2);
                        fc.vx = ff_sub(ff_mul(a, nvx), ff_mul(b, nx_));
                        fc.vy = ff_sub(ff_mul(a, nvy), ff_mul(b, ny_));
                        fc.vz = ff_sub(ff_mul(a, nvz), ff_mul(b, nz_));
                        vx = ff_to_d(fc.vx);
                        vy = ff_to_d(fc.vy);
                        vz = ff_to_d(fc.vz);
                    }
                    if (st.coated) r.f *= st.coat_t;
                }
            }
            r.x = x; r.y = y; r.z = z;
            r.vx = vx; r.vy = vy; r.vz = vz;
            fc.x = fx;
            fc.y = fy;
            fc.ok = true;
        } else {
            r.fail = true;
            r.vig = true;
        }
    }
    if (st.obsc_end > st.obsc_begin) {
        // src/batoid.cpp:169-171: vignetted |= contains(x, y), for every ray
        if (!have_f) {
            fx = fc.ok ? fc.x : d_to_ff(r.x);
            fy = fc.ok ? fc.y : d_to_ff(r.y);
        }
        // the common clear aperture, NOT(circle or annulus about the axis),
        // decided inline when the FP32 test is clear (ff_radius_less's first
        // step); everything else by the out-of-line postfix program
        int fast = -1;  // -1: not decided here; 0 / 1: obscured or not
        if (st.obsc_end - st.obsc_begin == 2) {
            const bt_obsc& o = P.obsc[st.obsc_begin];
            if (P.obsc[st.obsc_begin + 1].op == BT_O_NEGATION) {
                const float h2f = fmaf(fx.hi, fx.hi, fy.hi * fy.hi);
                // (positive radii tested on the integer pipe, as ff_radius_less)
                if (o.op == BT_O_CIRCLE && !d_nonzero(o.p[1]) && !d_nonzero(o.p[2]) &&
                    __double_as_longlong(o.p[0]) > 0) {
                    const float rf = ff_slot(&o.p[3]).hi, r2f = rf * rf;
                    if (h2f < r2f * (1.f - 1e-5f)) fast = 0;          // inside the circle: clear
                    else if (h2f > r2f * (1.f + 1e-5f)) fast = 1;     // outside: obscured
                } else if (o.op == BT_O_ANNULUS && !d_nonzero(o.p[2]) && !d_nonzero(o.p[3]) &&
                           __double_as_longlong(o.p[0]) > 0 && __double_as_longlong(o.p[1]) > 0) {
                    const float ri = ff_slot(&o.p[4]).hi, ro = ff_slot(&o.p[5]).hi;
                    const float ri2 = ri * ri, ro2 = ro * ro;
                    if (h2f > ri2 * (1.f + 1e-5f) && h2f < ro2 * (1.f - 1e-5f)) fast = 0;  // in the annulus
                    else if (h2f < ri2 * (1.f - 1e-5f) || h2f > ro2 * (1.f + 1e-5f)) fast = 1;
                }
            }
        }
        if (fast < 0) fast = ff_obsc_run(P, st.obsc_begin, st.obsc_end, fx, fy, r.x, r.y) ? 1 : 0;
        if (fast) r.vig = true;
    }
}
