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
__device__ __forceinline__ ff ff_horner_serial(ff x, const ff* c, int n) {
    ff r{0.f, 0.f};
    for (int i = n - 1; i >= 0; i--) r = ff_fma(r, x, c[i]);
    return r;
}

// The same as E(x^2) + x O(x^2) (even and odd coefficients): two
// independent Horner chains in x^2, half the dependent steps of one chain.
// The float-float chains are latency-bound, so the second chain is nearly
// free.  Rounding differs from the single chain at the ~1e-14 relative
// level of float-float arithmetic.
__device__ __forceinline__ ff ff_horner(ff x, const ff* c, int n) {
    if (n < 4) return ff_horner_serial(x, c, n);
    const ff x2 = ff_mul(x, x);
    ff e{0.f, 0.f}, o{0.f, 0.f};
    int i = n - 1;
    if ((i & 1) == 0) e = c[i--];
    for (; i >= 1; i -= 2) {
        o = ff_fma(o, x2, c[i]);
        e = ff_fma(e, x2, c[i - 1]);
    }
    return ff_fma(o, x, e);
}

// 2-D Horner with the reference's layout (row i: polynomial in y for x^i).
__device__ __forceinline__ ff ff_horner2d(ff x, ff y, const ff* c, int nx, int ny) {
    ff r{0.f, 0.f};
    for (int i = ny - 1; i >= 0; i--) r = ff_fma(r, x, ff_horner_serial(y, c + i * nx, nx));
    return r;
}

// The same over a triangular array (square, K = nx = ny, every coefficient
// with i + j >= K zero, as the Cartesian form of a Zernike sum): row i is
// evaluated over its K - i leading columns only.  The skipped terms are
// exact zeros, so the value is the full Horner's.
// Rows are taken in pairs (i, i - 1) whose Horner chains run interleaved in
// one loop (two independent dependency chains); every row and the outer
// recurrence are evaluated exactly as one row at a time would, so the value
// is unchanged.
__device__ __forceinline__ ff ff_horner2d_tri(ff x, ff y, const ff* c, int K) {
    ff r{0.f, 0.f};
    int i = K - 1;
    for (; i >= 1; i -= 2) {
        const int L = K - i;  // row i has L columns, row i - 1 has L + 1
        const ff* ca = c + i * K;
        const ff* cb = c + (i - 1) * K;
        ff a{0.f, 0.f}, b = cb[L];
        for (int j = L - 1; j >= 0; j--) {
            a = ff_fma(a, y, ca[j]);
            b = ff_fma(b, y, cb[j]);
        }
        r = ff_fma(ff_fma(r, x, a), x, b);
    }
    if (i == 0) r = ff_fma(r, x, ff_horner_serial(y, c, K));
    return r;
}

__device__ __forceinline__ float f_horner2d_tri(float x, float y, const ff* c, int K) {
    float r = 0.f;
    int i = K - 1;
    for (; i >= 1; i -= 2) {
        const int L = K - i;
        const ff* ca = c + i * K;
        const ff* cb = c + (i - 1) * K;
        float a = 0.f, b = cb[L].hi;
        for (int j = L - 1; j >= 0; j--) {
            a = fmaf(a, y, ca[j].hi);
            b = fmaf(b, y, cb[j].hi);
        }
        r = fmaf(fmaf(r, x, a), x, b);
    }
    if (i == 0) {
        float row = 0.f;
        for (int j = K - 1; j >= 0; j--) row = fmaf(row, y, c[j].hi);
        r = fmaf(r, x, row);
    }
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

// ---------------------------------------------------------------------------
// Float-float toolkit for the trace kernel.  On GB300 every FP64-pipe
// instruction -- DFMA, DADD, compares and double<->float conversions alike --
// occupies the pipe for the same time, and the FP32 pipe issues ~64 lanes
// for each FP64 lane, so the conversions below use integer and FP32
// instructions only.
// ---------------------------------------------------------------------------

__device__ __forceinline__ ff ff_make(float h, float l) { return ff{h, l}; }
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }

// Knuth's two-sum (no magnitude assumption).
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return ff{s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_add_f(ff a, float b) {
    const ff s = ff_two_sum(a.hi, b);
    const float e = s.lo + a.lo;
    const float h = s.hi + e;
    return ff{h, e - (h - s.hi)};
}

// a * b for float b, normalised.
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    const float p = a.hi * b;
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    const float s = p + e;
    return ff{s, e - (s - p)};
}

__device__ __forceinline__ ff ff_sqr(ff a) {
    const float p = a.hi * a.hi;
    float e = fmaf(a.hi, a.hi, -p);
    e = fmaf(2.f * a.hi, a.lo, e);
    const float s = p + e;
    return ff{s, e - (s - p)};
}

// a * b + c.
__device__ __forceinline__ ff ff_mad(ff a, ff b, ff c) { return ff_add(ff_mul(a, b), c); }

// Hardware approximations (PTX rcp.approx / sqrt.approx, relative error of
// a few 2^-23): starting points of the float-float corrections below, whose
// result error is then of the order of the square of the starting error.
__device__ __forceinline__ float f_rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float f_sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// a / b: a quotient estimate from the high parts, one correction from the
// float-float remainder a - q b.
__device__ __forceinline__ ff ff_div(ff a, ff b) {
    const float r = f_rcp_approx(b.hi);
    const float q1 = a.hi * r;
    // a - q1 * b, with the product q1 * b.hi exact
    const float p = q1 * b.hi;
    const float pe = fmaf(q1, b.hi, -p);
    const float d = ((a.hi - p) - pe) + (a.lo - q1 * b.lo);
    const float q2 = d * r;
    const float s = q1 + q2;
    return ff{s, q2 - (s - q1)};
}

// sqrt(a) (NaN for a < 0, 0 for 0): the FP32 root and one correction.
__device__ __forceinline__ ff ff_sqrt(ff a) {
    const float s = f_sqrt_approx(a.hi);
    if (!(a.hi > 0.f)) return ff{s, 0.f};
    const float e = fmaf(-s, s, a.hi) + a.lo;
    const float c = e * (0.5f * f_rcp_approx(s));
    const float h = s + c;
    return ff{h, c - (h - s)};
}

// 1 / sqrt(a): the FP32 estimate and one Newton step in float-float.
__device__ __forceinline__ ff ff_rsqrt(ff a) {
    const float y = rsqrtf(a.hi);
    // y (1 + (1 - a y^2) / 2)
    const ff ay2 = ff_mul_f(ff_mul_f(a, y), y);
    const float r = (1.f - ay2.hi) - ay2.lo;
    const float c = y * 0.5f * r;
    const float h = y + c;
    return ff{h, c - (h - y)};
}

// Signs and comparisons: for a normalised pair the sign is the high part's.
__device__ __forceinline__ bool ff_lt0(ff a) { return a.hi < 0.f; }
__device__ __forceinline__ bool ff_gt0(ff a) { return a.hi > 0.f; }
__device__ __forceinline__ bool ff_lt(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ float ff_abs_hi(ff a) { return fabsf(a.hi); }
__device__ __forceinline__ ff ff_abs(ff a) { return a.hi < 0.f ? ff_neg(a) : a; }

// float -> double, exact for normal floats, zeros, infinities and NaNs
// (FP32 subnormals become signed zeros), with integer instructions.
__device__ __forceinline__ double f2d_bits(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = (b >> 23) & 0xffu;
    const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
    const uint64_t man = (uint64_t)(b & 0x7fffffu) << 29;
    const uint64_t ed = (e == 0xffu) ? 0x7ffull : (uint64_t)(e + 896u);
    const uint64_t bits = (e == 0u) ? sign : (sign | (ed << 52) | man);
    return __longlong_as_double((long long)bits);
}

// Float-float to double: both parts exactly, one FP64 addition.
__device__ __forceinline__ double ff_to_d(ff a) { return f2d_bits(a.hi) + f2d_bits(a.lo); }

// Exact small unsigned integer (< 2^23) to float with one FP32 subtraction.
__device__ __forceinline__ float u23_to_f(uint32_t m) { return __uint_as_float(0x4b000000u | m) - 8388608.0f; }

// double -> float-float with integer and FP32 instructions.  hi holds the
// leading 24 bits (truncated), lo the remaining 29 bits rounded to 24: the
// pair equals d to ~2^-53 relative.  |d| below 2^-126 becomes a signed zero
// pair (below 2^-80 the low part is dropped); infinities and NaNs carry
// into hi.
__device__ __forceinline__ ff d_to_ff(double d) {
    const uint64_t b = (uint64_t)__double_as_longlong(d);
    const uint32_t hw = (uint32_t)(b >> 32);
    const uint32_t sign = hw & 0x80000000u;
    const int e = (int)((hw >> 20) & 0x7ffu);
    const uint32_t top = (uint32_t)((b >> 29) & 0x7fffffu);  // mantissa bits 51..29
    const uint32_t rest = (uint32_t)(b & 0x1fffffffu);       // mantissa bits 28..0
    float hi, lo;
    if (e >= 897 && e <= 1150) {
        hi = __uint_as_float(sign | ((uint32_t)(e - 896) << 23) | top);
        // rest * 2^(e - 1075), rest < 2^29 split into 23 + 6 bits
        const float r = fmaf(u23_to_f(rest >> 6), 64.f, u23_to_f(rest & 63u));
        const int se = e - 1075 + 127;
        const float scale = (se >= 1) ? __uint_as_float(sign | ((uint32_t)se << 23)) : 0.f;
        lo = r * scale;
    } else if (e == 0x7ff) {
        hi = __uint_as_float(sign | 0x7f800000u | top | ((rest != 0u) ? 1u : 0u));
        lo = 0.f;
    } else if (e > 1150) {
        hi = __uint_as_float(sign | 0x7f800000u);  // beyond float range
        lo = 0.f;
    } else {
        hi = __uint_as_float(sign);
        lo = 0.f;
    }
    // renormalise (lo may reach ulp(hi))
    const float s = hi + lo;
    return (e >= 897 && e <= 1150) ? ff{s, lo - (s - hi)} : ff{hi, lo};
}

// A float-float pair packed by the host into one double slot.
__device__ __forceinline__ ff ff_slot(const double* p) { return *reinterpret_cast<const ff*>(p); }
