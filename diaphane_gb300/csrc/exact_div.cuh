// Correctly rounded f32 division n / d for finite d >= 1 (here d = 1 + loss,
// loss >= 0), without the library division's slow path for zero and tiny
// numerators.
//
// The library's IEEE division is correct for every input but takes a slow
// path when the numerator is zero or very small — measured 3x (zero) to 7x
// (subnormal) the cost of a normal division on GB300.  Absorbing-layer cells
// are exactly zero until a wave reaches them and decay through tiny values
// after it leaves, so a step spent roughly twice as long as it needed to
// while the grid was partly empty.  This wrapper keeps the library division
// for normal numerators and handles the rest exactly:
//   * ±0 / d = ±0 for d > 0;
//   * |n| < 2^-100: n·2^64 is exact, its quotient q is normal and computed on
//     the fast path; if q·2^-64 is normal the scaling is exact.  Otherwise the
//     result lies on the subnormal grid (spacing 2^-149, i.e. 2^-85 before
//     scaling back): q is rounded to that grid, and when q sits exactly on a
//     grid midpoint the sign of the exact remainder r = n·2^64 - q·d (one
//     FMA, exact) decides the direction, as in the standard
//     remainder-corrected rounding of a quotient (Markstein; Muller et al.,
//     Handbook of Floating-Point Arithmetic, ch. 4).  q's own ulp is at most
//     2^-86 there, so every grid midpoint is representable and only an exact
//     midpoint needs the remainder.
// The result equals the IEEE quotient bit for bit (checked against the
// library division on random and edge-case inputs by the test suite).
#pragma once

namespace diaphane {

// Numerators the library division handles on its fast path (measured: the
// cost steps up between 2^-100 and 2^-110 and for zero), plus inf and NaN,
// which exact_div hands to the library anyway.
__device__ __forceinline__ bool plain_division_is_fast(float n) { return !(fabsf(n) < 0x1p-100f); }

// The subnormal-quotient case of exact_div, out of line (it is rare, and
// inlining it at every division site costs instruction-cache misses).  q is
// the correctly rounded quotient of ns = n·2^64 by d, |q| < 2^-62.
static __device__ __noinline__ float exact_div_subnormal(float n, float ns, float d, float q) {
    const float r = fmaf(-q, d, ns);
    const float u = q * 0x1p85f; // in units of the subnormal spacing; |u| < 2^23, exact
    const float f = floorf(u);
    float k;
    if (u - f == 0.5f) k = r > 0.0f ? f + 1.0f : (r < 0.0f ? f : rintf(u));
    else k = rintf(u);
    return copysignf(k * 0x1p-149f, n);
}

// exact_div without branches on the common paths: a tiny numerator is scaled
// by 2^64 (exact), a zero one is swapped for 1, one fast-path division is
// done, and the quotient is scaled or selected back.  Only a quotient that
// lands in the subnormal range takes the out-of-line fixup.
__device__ __forceinline__ float exact_div(float n, float d) {
    const bool fast = plain_division_is_fast(n);
    const bool zero = n == 0.0f;
    const float ns = fast ? n : n * 0x1p64f;
    const float q = (zero ? 1.0f : ns) / d;
    if (fast || zero) return zero ? n : q;
    if (fabsf(q) >= 0x1p-62f) return q * 0x1p-64f;
    return exact_div_subnormal(n, ns, d, q);
}

} // namespace diaphane
