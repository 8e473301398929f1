// Float-float ("double-single") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats, |lo| <= ulp(hi)/2,
// giving ~44-48 significant bits.  The error-free transformations are the
// classic ones: Knuth's two-sum and the FMA-based two-product (Dekker's
// product with a fused multiply-add).  On GB300 the FP32 pipe issues 64
// lanes for every FP64 lane, so a float-float multiply-add (~14 FP32
// instructions) is several times cheaper than one FP64 FMA.
//
// Used for polynomial perturbation terms whose magnitude is small compared
// with the result they are added to (asphere polynomials, Zernike / Cartesian
// polynomial surfaces): there ~44 bits relative to the term is far below the
// 1e-12 m position tolerance.
#pragma once

struct ff {
    float hi;
    float lo;
};

__device__ __forceinline__ ff ff_from(double d) {
    const float h = __double2float_rn(d);
    return ff{h, __double2float_rn(d - (double)h)};
}

__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

// a * b with both operands float-float.
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    const float s = p + e;
    return ff{s, e - (s - p)};
}

// a + b (two-sum on the high parts, low parts added to the error).
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    float err = (a.hi - (s - bb)) + (b.hi - bb);
    err += a.lo + b.lo;
    const float h = s + err;
    return ff{h, err - (h - s)};
}

// r * x + c, the Horner step.
__device__ __forceinline__ ff ff_fma(ff r, ff x, ff c) { return ff_add(ff_mul(r, x), c); }

// Coefficient arrays are stored as (hi, lo) float pairs in the double pool.
__device__ __forceinline__ const ff* ff_ptr(const double* pool, int off) {
    return reinterpret_cast<const ff*>(pool + off);
}

// Horner in one variable: sum_{i<n} c[i] x^i.
__device__ __forceinline__ ff ff_horner(ff x, const ff* c, int n) {
    ff r{0.f, 0.f};
    for (int i = n - 1; i >= 0; i--) r = ff_fma(r, x, c[i]);
    return r;
}

// 2-D Horner with the reference's layout (row i: polynomial in y for x^i).
__device__ __forceinline__ ff ff_horner2d(ff x, ff y, const ff* c, int nx, int ny) {
    ff r{0.f, 0.f};
    for (int i = ny - 1; i >= 0; i--) r = ff_fma(r, x, ff_horner(y, c + i * nx, nx));
    return r;
}

// Plain FP32 Horner on the high parts (for Newton derivatives).
__device__ __forceinline__ float f_horner2d(float x, float y, const ff* c, int nx, int ny) {
    float r = 0.f;
    for (int i = ny - 1; i >= 0; i--) {
        float row = 0.f;
        for (int j = nx - 1; j >= 0; j--) row = fmaf(row, y, c[i * nx + j].hi);
        r = fmaf(r, x, row);
    }
    return r;
}
