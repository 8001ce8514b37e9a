// Device-side scalar helpers with the reference's exact semantics.
//
// Every kernel is compiled with -fmad=false and IEEE division/sqrt, so
// `a * b + c` is two rounded operations, as glam (which never fuses) does.
// One thread evaluates one lane of the reference's 4-wide SIMD code.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace swr {

// Rust `f32 as i32`: truncate, saturate, NaN -> 0 (cvt.rzi.s32.f32).
__device__ __forceinline__ int32_t f2i_sat(float x) { return __float2int_rz(x); }
// Rust `f32 as u32`: truncate, saturate (negatives -> 0), NaN -> 0.
__device__ __forceinline__ uint32_t f2u_sat(float x) { return __float2uint_rz(x); }
// Rust `f32 as u8`.
__device__ __forceinline__ uint32_t f2u8_sat(float x) {
    uint32_t u = __float2uint_rz(x);
    return u > 255u ? 255u : u;
}
__device__ __forceinline__ float i2f(int32_t i) { return __int2float_rn(i); }
__device__ __forceinline__ float u2f(uint32_t i) { return __uint2float_rn(i); }

// f32::round: nearest, ties away from zero. x - trunc(x) is exact.
__device__ __forceinline__ float round_away(float x) {
    float t = truncf(x);
    float d = x - t;
    if (fabsf(d) >= 0.5f) t += copysignf(1.0f, x);
    return t;
}

// Wrapping i32 arithmetic (Rust release builds wrap).
__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
__device__ __forceinline__ int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
__device__ __forceinline__ int32_t wabs(int32_t a) { return a < 0 ? (int32_t)(0u - (uint32_t)a) : a; }

// Depth key: orderable(z) in the high word, ~(seq8 + 1) in the low word, so
// an unsigned minimum picks the smallest z and, among equal z, the largest
// canonical sequence number (the last packet a sequential depth test
// `z <= current` would have accepted). -0 and +0 compare equal in the
// reference, so -0 is canonicalised to +0.
__device__ __forceinline__ uint32_t float_to_ordered(float f) {
    uint32_t b = __float_as_uint(f);
    if (f == 0.0f) b = 0u;
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ordered_to_float(uint32_t o) {
    uint32_t b = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
    return __uint_as_float(b);
}
__device__ __forceinline__ unsigned long long make_key(float z, uint32_t seq8) {
    return ((unsigned long long)float_to_ordered(z) << 32) | (unsigned long long)(0xFFFFFFFEu - seq8);
}
__device__ __forceinline__ uint32_t key_seq8(unsigned long long k) {
    return 0xFFFFFFFEu - (uint32_t)(k & 0xFFFFFFFFull);
}

// --- reciprocal square root ------------------------------------------
//
// IEEE mode: 1 / sqrt(x), two correctly rounded operations
// (src/math.rs:46-49).
__device__ __forceinline__ float rsqrt_ieee(float x) { return __fdiv_rn(1.0f, __fsqrt_rn(x)); }

// FRSQRTE (single precision, FPCR.AH = 0): 8-bit estimate from the Arm
// architecture's RecipSqrtEstimate, table-driven. `tab` holds estimate<7:0>
// for the 9-bit scaled operand (128..511).
static __device__ __noinline__ float frsqrte_special(float x, const uint8_t* tab) {
    const uint32_t b = __float_as_uint(x);
    if (x != x) return __uint_as_float(b | 0x00400000u);
    if (x == 0.0f) return __uint_as_float((b & 0x80000000u) | 0x7F800000u);
    if (b & 0x80000000u) return __uint_as_float(0x7FC00000u);
    if (b == 0x7F800000u) return 0.0f;
    int32_t e = (int32_t)((b >> 23) & 0xFFu);
    uint64_t frac = (uint64_t)(b & 0x7FFFFFu) << 29;  // fraction<51:0>
    if (e == 0) {
        while (((frac >> 51) & 1ull) == 0ull) {
            frac <<= 1;
            e -= 1;
        }
        frac = (frac << 1) & ((1ull << 52) - 1ull);
    }
    uint32_t scaled;
    if ((e & 1) == 0)
        scaled = 256u | (uint32_t)(frac >> 44);
    else
        scaled = 128u | (uint32_t)(frac >> 45);
    const int32_t rexp = (380 - e) / 2;
    const uint32_t est = tab[scaled];
    return __uint_as_float(((uint32_t)(rexp & 0xFF) << 23) | (est << 15));
}
__device__ __forceinline__ float frsqrte(float x, const uint8_t* tab) {
    const uint32_t b = __float_as_uint(x);
    const uint32_t e = b >> 23;  // sign bit included: negative inputs leave the fast path
    if (e - 1u < 254u) {         // positive normal: fraction<51:44> / <51:45> are mantissa bits
        const uint32_t m = b & 0x7FFFFFu;
        const uint32_t scaled = (e & 1u) ? (128u | (m >> 16)) : (256u | (m >> 15));
        const uint32_t rexp = (380u - e) >> 1;
        return __uint_as_float((rexp << 23) | ((uint32_t)tab[scaled] << 15));
    }
    return frsqrte_special(x, tab);
}
// FRSQRTS: (3 - a*b) / 2 with a single rounding.
__device__ __forceinline__ float frsqrts(float a, float b) {
    if (isfinite(a) && isfinite(b)) return __fmul_rn(__fmaf_rn(-a, b, 3.0f), 0.5f);
    if (a != a) return a;
    if (b != b) return b;
    const bool ia = isinf(a), ib = isinf(b);
    if ((ia && b == 0.0f) || (a == 0.0f && ib)) return 1.5f;
    if (ia || ib) {
        const uint32_t s = (__float_as_uint(a) ^ __float_as_uint(b) ^ 0x80000000u) & 0x80000000u;
        return __uint_as_float(s | 0x7F800000u);
    }
    return __fmul_rn(__fmaf_rn(-a, b, 3.0f), 0.5f);
}
// src/math.rs:17-25: y0 = vrsqrteq(x); y1 = y0 * vrsqrtsq(x * y0, y0).
// For a positive normal x the estimate y0 is a positive normal and x * y0
// (about sqrt(x)) is finite, so FRSQRTS takes its finite branch: that path
// is evaluated inline, the rest goes through the general functions.
__device__ __forceinline__ float rsqrt_aarch64(float x, const uint8_t* tab) {
    const uint32_t b = __float_as_uint(x);
    const uint32_t e = b >> 23;
    if (e - 1u < 254u) {
        const uint32_t m = b & 0x7FFFFFu;
        const uint32_t scaled = (e & 1u) ? (128u | (m >> 16)) : (256u | (m >> 15));
        const float y0 = __uint_as_float((((380u - e) >> 1) << 23) | ((uint32_t)tab[scaled] << 15));
        return __fmul_rn(y0, __fmul_rn(__fmaf_rn(-__fmul_rn(x, y0), y0, 3.0f), 0.5f));
    }
    const float y0 = frsqrte(x, tab);
    return __fmul_rn(y0, frsqrts(__fmul_rn(x, y0), y0));
}
__device__ __forceinline__ float rsqrt_mode(float x, uint32_t mode, const uint8_t* tab) {
    return mode == 1u ? rsqrt_aarch64(x, tab) : rsqrt_ieee(x);
}

}  // namespace swr
