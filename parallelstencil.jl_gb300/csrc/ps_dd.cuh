// ps_dd.cuh -- FP64 values as pairs of FP32 numbers (h + l, a 47-bit significand) for GB300,
// whose FP32 and integer pipes issue 128 instructions / clk / SM against 2 for FP64 (and for
// f64 <-> f32 conversions): splitting uses integer bit operations only, sums an exact two-sum of
// the high parts, products FMA to recover the rounding error of h*h.
#pragma once

namespace ps {

struct dd {
    float h, l;
};

// Split a double into two floats with integer operations only (see file comment).
__device__ __forceinline__ dd dd_split(double x, bool& big) {
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const unsigned t = hw & 0x7FFFFFFFu;
    const unsigned sgn = hw & 0x80000000u;
    // high part: sign | (e - 896) << 23 | top 23 mantissa bits (truncated), for e in [897, 1150]
    const unsigned fb = __funnelshift_l(lw, hw, 3) ^ 0x40000000u;
    float h = __uint_as_float((fb & 0x7FFFFFFFu) | sgn);
    // low part: the next 23 mantissa bits m, as m * 2^(e - 1069), for e >= 943
    const float m = __uint_as_float(((lw >> 6) & 0x7FFFFFu) | 0x4B000000u) - 8388608.0f;
    const unsigned sb = (((hw << 3) & 0xFF800000u) - 0xD7000000u) | sgn;
    float l = m * __uint_as_float(sb);
    h = t < 0x38100000u ? 0.0f : h;  // e < 897: below FP32's normal range
    l = t < 0x3AF00000u ? 0.0f : l;  // e < 943: keep the 24-bit high part only
    big |= t >= 0x47F00000u;         // e >= 1151: outside FP32's range (or inf / nan)
    return {h, l};
}

// Exact conversion of a float to double with integer operations (zero and denormals -> ±0 / tiny).
__device__ __forceinline__ double f32_to_f64(float f) {
    const unsigned b = __float_as_uint(f);
    unsigned hi = (((b >> 3) & 0x0FFFFFFFu) + 0x38000000u) | (b & 0x80000000u);
    hi = (b & 0x7F800000u) ? hi : (b & 0x80000000u);
    return __hiloint2double((int)hi, (int)(b << 29));
}

__device__ __forceinline__ dd dd_add(dd a, dd b) {
    const float s = a.h + b.h;
    const float bb = s - a.h;
    const float e = (a.h - (s - bb)) + (b.h - bb);
    return {s, e + (a.l + b.l)};
}
__device__ __forceinline__ dd dd_sub(dd a, dd b) { return dd_add(a, dd{-b.h, -b.l}); }
__device__ __forceinline__ dd dd_mul(dd a, dd b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return {p, e};
}

// x * 2^k for a power-of-two float factor (exact unless the result leaves FP32's range)
__device__ __forceinline__ dd dd_scale(dd a, float p2) { return {a.h * p2, a.l * p2}; }

}  // namespace ps
