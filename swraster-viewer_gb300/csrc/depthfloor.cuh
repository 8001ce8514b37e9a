// Depth floor of a raster packet, for the raster's occlusion culling: a lower
// bound of every depth the raster's own arithmetic can produce for a covered
// lane of the packet. The same source compiles for the device (directed-
// rounding intrinsics) and for the host (directed rounding obtained from
// error-free transformations of round-to-nearest results), so the bound can be
// checked on a CPU against an exhaustive walk of the packet.
//
// The floor covers every rounding of the raster's arithmetic (u = 2^-24):
//  - edge values: the origin evaluation (a x + b y) + c and at most 16
//    sequential additions err by at most 24u (|a| X + |b| Y + |c| +
//    256 (|a| + |b|)) per edge, X and Y the largest sample coordinates. A
//    covered lane has all three computed edge values >= 0 and the exact values
//    sum to the doubled area A plus top-left biases (<= 0), so b1, b2 >= 0 and
//    b1 + b2 <= B = (1 + (sum of the three errors) / A)(1 + u)^3;
//  - zi and oi are three-term sums, within EZ = 5u (|Z0| + B |D1| + B |D2|)
//    (EO likewise) of the exact affine values, and z = zi * (1 / oi) adds two
//    roundings;
//  - (exact zi - EZ) / (exact oi +- EO) is a ratio of affine functions of
//    (b1, b2) with a positive denominator, so its minimum over the triangle
//    {b1, b2 >= 0, b1 + b2 <= B} is at a corner; corners are evaluated with
//    directed rounding.
// No floor is taken (false) when the packet's int32 setup arithmetic could
// have wrapped, when its 1/w interpolant could reach 0, for non-finite inputs,
// or when B would exceed about 1.28.
#pragma once

#include <cfloat>
#include <cmath>
#include <cstdint>

namespace swr {

constexpr float kUlp24 = 5.9604645e-8f;  // 2^-24

#ifdef __CUDA_ARCH__
__device__ __forceinline__ float df_add_rd(float a, float b) { return __fadd_rd(a, b); }
__device__ __forceinline__ float df_add_ru(float a, float b) { return __fadd_ru(a, b); }
__device__ __forceinline__ float df_sub_rd(float a, float b) { return __fsub_rd(a, b); }
__device__ __forceinline__ float df_mul_rd(float a, float b) { return __fmul_rd(a, b); }
__device__ __forceinline__ float df_mul_ru(float a, float b) { return __fmul_ru(a, b); }
__device__ __forceinline__ float df_div_rd(float a, float b) { return __fdiv_rd(a, b); }
__device__ __forceinline__ bool df_finite(float x) { return isfinite(x); }
#else
// Round-to-nearest result s of a + b, moved one float down (up) when the
// exact sum lies below (above) it; the exact error comes from TwoSum.
inline float df_sum_dir(float a, float b, bool up) {
    const float s = a + b;
    if (!std::isfinite(s)) {
        if (!std::isfinite(a) || !std::isfinite(b)) return s;
        return s > 0.0f ? (up ? s : FLT_MAX) : (up ? -FLT_MAX : s);
    }
    const float bb = s - a;
    const float err = (a - (s - bb)) + (b - bb);
    if (up) return err > 0.0f ? std::nextafter(s, INFINITY) : s;
    return err < 0.0f ? std::nextafter(s, -INFINITY) : s;
}
// Product: the exact error a b - p is fma(a, b, -p).
inline float df_prod_dir(float a, float b, bool up) {
    const float p = a * b;
    if (!std::isfinite(p)) {
        if (!std::isfinite(a) || !std::isfinite(b)) return p;
        return p > 0.0f ? (up ? p : FLT_MAX) : (up ? -FLT_MAX : p);
    }
    const float err = std::fma(a, b, -p);
    if (up) return err > 0.0f ? std::nextafter(p, INFINITY) : p;
    return err < 0.0f ? std::nextafter(p, -INFINITY) : p;
}
inline float df_add_rd(float a, float b) { return df_sum_dir(a, b, false); }
inline float df_add_ru(float a, float b) { return df_sum_dir(a, b, true); }
inline float df_sub_rd(float a, float b) { return df_sum_dir(a, -b, false); }
inline float df_mul_rd(float a, float b) { return df_prod_dir(a, b, false); }
inline float df_mul_ru(float a, float b) { return df_prod_dir(a, b, true); }
// Quotient: a - q b = fma(-q, b, a) exactly, and a / b - q has its sign
// times the sign of b.
inline float df_div_rd(float a, float b) {
    const float q = a / b;
    if (!std::isfinite(q)) {
        if (!std::isfinite(a) || !std::isfinite(b) || b == 0.0f) return q;
        return q > 0.0f ? FLT_MAX : q;
    }
    const float r = std::fma(-q, b, a);
    const bool below = (r < 0.0f && b > 0.0f) || (r > 0.0f && b < 0.0f);
    return below ? std::nextafter(q, -INFINITY) : q;
}
inline bool df_finite(float x) { return std::isfinite(x); }
#endif

// Error bound of one edge's computed values over the packet (false: the
// edge's integer terms could have wrapped or lost exactness).
__host__ __device__ __forceinline__ bool edge_error(long long xi, long long yi, long long xj, long long yj, float X,
                                                    float Y, float& err) {
    const long long a = yj - yi, b = xi - xj, c = xj * yi - xi * yj;
    const long long lim = 1ll << 24, climb = (1ll << 31) - 2;
    if (a > lim || a < -lim || b > lim || b < -lim || c > climb || c < -climb) return false;
    const float fa = fabsf((float)a), fb = fabsf((float)b), fc = fabsf((float)c) + 1.0f;
    err = (32.0f * kUlp24) * (((fa * X + fb * Y) + fc) + 256.0f * (fa + fb));
    return true;
}

// Lower bound of every depth the raster computes for a covered lane of a
// packet with subpixel vertices p (x0, y0, x1, y1, x2, y2), depth and 1/w
// interpolants zow and oow (value at vertex 0, then differences to vertices
// 1 and 2) and sample coordinates below xe + 32 and ye + 32 (subpixels, xe and
// ye the end of the packet's rect clipped to its 64-px tile); false when no
// bound is taken.
__host__ __device__ inline bool depth_floor(const int32_t p[6], const float zow[3], const float oow[3], int32_t xe,
                                            int32_t ye, float& zlo) {
#pragma unroll
    for (int i = 0; i < 6; ++i)
        if (p[i] > (1 << 28) || p[i] < -(1 << 28)) return false;
    const long long x0 = p[0], y0 = p[1], x1 = p[2], y1 = p[3], x2 = p[4], y2 = p[5];
    const long long area = (x1 - x0) * (y2 - y0) - (x2 - x0) * (y1 - y0);
    if (area >= 0 || area <= -(1ll << 31)) return false;
    const float X = (float)(xe + 32), Y = (float)(ye + 32);
    float e12, e20, e01;
    if (!edge_error(x1, y1, x2, y2, X, Y, e12) || !edge_error(x2, y2, x0, y0, X, Y, e20) ||
        !edge_error(x0, y0, x1, y1, X, Y, e01))
        return false;
    const float A = (float)(-area) * (1.0f - 2.0f * kUlp24);
    const float rel = ((e12 + e20) + e01) / A;
    if (!(rel < 0.25f)) return false;
    const float B = df_add_ru(1.0f, df_mul_ru(rel + 8.0f * kUlp24, 1.125f));
    const float Z0 = zow[0], D1 = zow[1], D2 = zow[2];
    const float O0 = oow[0], P1 = oow[1], P2 = oow[2];
    if (!(df_finite(Z0) && df_finite(D1) && df_finite(D2) && df_finite(O0) && df_finite(P1) && df_finite(P2)))
        return false;
    const float EZ = (5.0f * kUlp24) * (fabsf(Z0) + B * (fabsf(D1) + fabsf(D2))) + 1e-30f;
    const float EO = (5.0f * kUlp24) * (fabsf(O0) + B * (fabsf(P1) + fabsf(P2))) + 1e-30f;
    if (!(df_finite(EZ) && df_finite(EO))) return false;
    float lo = INFINITY;
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        const float dz = v == 1 ? D1 : D2, dw = v == 1 ? P1 : P2;
        const float zc = v == 0 ? Z0 : df_add_rd(Z0, df_mul_rd(B, dz));
        const float wlo = v == 0 ? O0 : df_add_rd(O0, df_mul_rd(B, dw));
        const float whi = v == 0 ? O0 : df_add_ru(O0, df_mul_ru(B, dw));
        const float n = df_sub_rd(zc, EZ);
        const float dlo = df_sub_rd(wlo, EO), dhi = df_add_ru(whi, EO);
        if (!(dlo > 0.0f) || !df_finite(n)) return false;
        lo = fminf(lo, fminf(df_div_rd(n, dhi), df_div_rd(n, dlo)));
    }
    lo = lo >= 0.0f ? df_mul_rd(lo, 1.0f - 4.0f * kUlp24) : df_mul_rd(lo, 1.0f + 4.0f * kUlp24);
    zlo = df_sub_rd(lo, 1e-30f);
    return zlo == zlo;
}

}  // namespace swr
